// ref_emul.cpp -- runs the reference's own column-major tile bodies on the CPU
// (through ref_shim.h) to produce golden outputs.  Test infrastructure only.
//
// The tile bodies are included from the reference sources at build time (see
// oracle/ref_emul/Makefile); no reference source is copied into this project.
// Only the bodies the reference computes as a correct column-major GEMM are
// exposed:
//   fw_128_32x32   CUDA/framework/kernel_128_new.h:131  (framework strategy 2)
//   li_256_*       CUDA/batching/kernel_256.h:1,55,114,195,312,428  (b = 1)
//   li_128_*       CUDA/batching/kernel_128.h:1,63,135,256,439
// Each body computes C += A*B (alpha = beta = 1) for column-major A (ld = M),
// B (ld = K), C (ld = M) with M, N multiples of the tile and K a multiple of
// the k-stage.
//
// Usage: ref_emul <kernel> <in.bin> <out.bin>
//   in.bin : int32 M, N, K, then float32 A[M*K], B[K*N], C[M*N]
//   out.bin: float32 C[M*N] after one launch over the whole (M/tm, N/tn) grid
#include "ref_shim.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

thread_local dim3 threadIdx;
thread_local dim3 blockIdx;
thread_local std::barrier<>* g_block_barrier = nullptr;

namespace fw {
inline float fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
#include REF_FW_KERNEL_128_NEW
}  // namespace fw

namespace li {
inline float fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
#include REF_LI_KERNEL_256
#include REF_LI_KERNEL_128
}  // namespace li

struct Body {
  const char* name;
  int threads, tm, tn, kstage;
  // (M, N, K, A, B, C, block_base_m, block_base_n, sh)
  std::function<void(int, int, int, float*, float*, float*, int, int, float*)> run;
};

static std::vector<Body> bodies() {
  using namespace std::placeholders;
  std::vector<Body> v;
  v.push_back({"fw_128_32x32", 128, 32, 32, 8,
               [](int M, int N, int K, float* A, float* B, float* C, int, int, float* sh) {
                 fw::gemm_128_32x32(M, N, K, A, B, C, sh);
               }});
#define LI256(TM, TN, KS)                                                                  \
  v.push_back({"li_256_" #TM "x" #TN, 256, TM, TN, KS,                                     \
               [](int M, int N, int K, float* A, float* B, float* C, int bm, int bn,       \
                  float* sh) { li::gemm_256_##TM##x##TN(M, N, K, A, B, C, bm, bn, sh); }});
  LI256(16, 16, 16)
  LI256(32, 32, 8)
  LI256(64, 64, 8)
  LI256(128, 64, 8)
  LI256(64, 128, 8)
  LI256(128, 128, 8)
#undef LI256
#define LI128(TM, TN)                                                                       \
  v.push_back({"li_128_" #TM "x" #TN, 128, TM, TN, 8,                                       \
               [](int M, int N, int K, float* A, float* B, float* C, int, int, float* sh) { \
                 li::gemm_128_##TM##x##TN(M, N, K, A, B, C, sh);                            \
               }});
  LI128(16, 16)
  LI128(32, 32)
  LI128(64, 64)
  LI128(64, 128)
  LI128(128, 64)
#undef LI128
  return v;
}

int main(int argc, char** argv) {
  if (argc == 2 && std::string(argv[1]) == "--list") {
    for (auto& b : bodies())
      std::printf("%s %d %d %d %d\n", b.name, b.threads, b.tm, b.tn, b.kstage);
    return 0;
  }
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s <kernel>|--list <in.bin> <out.bin>\n", argv[0]);
    return 2;
  }
  const Body* body = nullptr;
  static std::vector<Body> all = bodies();
  for (auto& b : all)
    if (std::string(argv[1]) == b.name) body = &b;
  if (!body) { std::fprintf(stderr, "unknown kernel %s\n", argv[1]); return 2; }

  FILE* f = std::fopen(argv[2], "rb");
  if (!f) { std::perror("in"); return 2; }
  int32_t dims[3];
  if (std::fread(dims, 4, 3, f) != 3) return 2;
  const int M = dims[0], N = dims[1], K = dims[2];
  if (M % body->tm || N % body->tn || K % body->kstage || M <= 0 || N <= 0 || K <= 0) {
    std::fprintf(stderr, "shape %dx%dx%d not supported by %s\n", M, N, K, body->name);
    return 2;
  }
  // Guard bands of NaN after every operand catch any read past the matrix.
  const size_t pad = 1024;
  std::vector<float> A((size_t)M * K + pad, __builtin_nanf("")), B((size_t)K * N + pad, __builtin_nanf("")),
      C((size_t)M * N + pad, __builtin_nanf(""));
  if (std::fread(A.data(), 4, (size_t)M * K, f) != (size_t)M * K) return 2;
  if (std::fread(B.data(), 4, (size_t)K * N, f) != (size_t)K * N) return 2;
  if (std::fread(C.data(), 4, (size_t)M * N, f) != (size_t)M * N) return 2;
  std::fclose(f);

  std::vector<float> sh(4 * 128 * 8);
  for (int bx = 0; bx < M / body->tm; ++bx) {
    for (int by = 0; by < N / body->tn; ++by) {
      std::fill(sh.begin(), sh.end(), __builtin_nanf(""));
      std::barrier<> bar(body->threads);
      std::vector<std::thread> th;
      th.reserve(body->threads);
      for (int t = 0; t < body->threads; ++t) {
        th.emplace_back([&, t] {
          threadIdx.x = t;
          blockIdx.x = bx;
          blockIdx.y = by;
          g_block_barrier = &bar;
          body->run(M, N, K, A.data(), B.data(), C.data(), bx * body->tm, by * body->tn, sh.data());
          bar.arrive_and_drop();
        });
      }
      for (auto& x : th) x.join();
    }
  }
  for (size_t i = (size_t)M * N; i < C.size(); ++i)
    if (!__builtin_isnan(C[i])) { std::fprintf(stderr, "write past C\n"); return 3; }
  FILE* o = std::fopen(argv[3], "wb");
  if (!o) { std::perror("out"); return 2; }
  std::fwrite(C.data(), 4, (size_t)M * N, o);
  std::fclose(o);
  return 0;
}
