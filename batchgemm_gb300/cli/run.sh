#!/bin/bash
# Sweep of the reference framework's run script (CUDA/framework/run.sh) on
# bgemm_gemm: batch sizes 8 .. 256 of the shape file, thresholds 512 / 6000,
# log lines appended to log-test-verify3.  Run it from a directory whose
# ../data holds data_MN_K_512_128, or pass the shape file as $1.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
exe="$here/../bgemm_gemm"
data="${1:-../data/data_MN_K_512_128}"
mode="${2:-simt}"
threshold=512
TLP=6000
rm -f log-test-verify3
for B in 8 16 32 64 128 256; do
  "$exe" $B $threshold $TLP --data "$data" --mode "$mode" >> log-test-verify3
done
echo "ok==================================" >> log-test-verify3
