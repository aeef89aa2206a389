"""Generates the golden fixtures in this folder from the reference itself.

Run in a checkout that has the reference next to it:

    python tests/golden/gen_golden.py [--ref <reference checkout>]

It writes
  * ``ref_kernels.npz`` -- seeded inputs and the outputs of the reference's own
    column-major tile bodies (CUDA/framework/kernel_128_new.h:131,
    CUDA/batching/kernel_256.h, CUDA/batching/kernel_128.h), run on the CPU by
    ``oracle/_ref/ref_emul`` (compiled from the reference sources by
    ``oracle/ref_emul/Makefile``).  Each tile body computes C += A*B
    column-major, so the outputs pin the oracle's in-place FP32 chain bit for bit.
  * ``ref_dataset_shapes.npy`` -- the (M, N, K) rows of the reference's shape
    fixture CUDA/data/data_MN_K_512_128 (read as ``fs >> M >> N >> K`` in
    CUDA/framework/gemm.cu:39-41); the first B rows are the reference's batch
    of size B.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

# (kernel, M, N, K): every shape is a multiple of the body's tile and k-stage.
CASES = [
    ("fw_128_32x32", 64, 96, 40),
    ("fw_128_32x32", 32, 32, 8),
    ("li_256_16x16", 48, 32, 48),
    ("li_256_32x32", 64, 64, 24),
    ("li_256_64x64", 128, 64, 16),
    ("li_256_128x64", 128, 128, 16),
    ("li_256_64x128", 64, 128, 24),
    ("li_256_128x128", 128, 128, 16),
    ("li_128_16x16", 32, 48, 16),
    ("li_128_32x32", 64, 32, 32),
    ("li_128_64x64", 64, 128, 16),
    ("li_128_64x128", 64, 128, 8),
    ("li_128_128x64", 128, 64, 16),
]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=oracle.reference_root())
    args = ap.parse_args()
    exe = oracle.build_ref_emul(args.ref)
    if exe is None:
        sys.exit("reference checkout not found at %s" % args.ref)
    rng = np.random.default_rng(20240607)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for i, (kern, M, N, K) in enumerate(CASES):
            A = rng.uniform(-1, 1, M * K).astype(np.float32)
            B = rng.uniform(-1, 1, K * N).astype(np.float32)
            C0 = rng.uniform(-1, 1, M * N).astype(np.float32)
            fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
            with open(fin, "wb") as f:
                np.array([M, N, K], np.int32).tofile(f)
                A.tofile(f)
                B.tofile(f)
                C0.tofile(f)
            subprocess.run([exe, kern, fin, fout], check=True)
            C = np.fromfile(fout, np.float32)
            assert C.size == M * N
            p = "c%02d_" % i
            out[p + "kernel"] = np.array(kern)
            out[p + "mnk"] = np.array([M, N, K], np.int32)
            out[p + "A"], out[p + "B"], out[p + "C0"], out[p + "C"] = A, B, C0, C
    out["ncases"] = np.array(len(CASES), np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), **out)

    shapes = np.loadtxt(os.path.join(args.ref, "CUDA", "data", "data_MN_K_512_128"),
                        dtype=np.int32).reshape(-1, 3)
    np.save(os.path.join(HERE, "ref_dataset_shapes.npy"), shapes.astype(np.int16))
    print("wrote %d kernel cases, %d dataset rows" % (len(CASES), shapes.shape[0]))


if __name__ == "__main__":
    main()
