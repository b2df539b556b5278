// Shared helpers of the pplacer_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <string>

#include "../../include/pplacer_gb300.h"

namespace pgb {

// Last error of the calling host thread (pgb_last_error).
void set_error(const char *fmt, ...);
extern std::atomic<uint64_t> g_launches;

inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define PGB_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) {                                                              \
      ::pgb::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
      return PGB_ERR_CUDA;                                                                \
    }                                                                                     \
  } while (0)

#define PGB_LAUNCH_CHECK()                                                                 \
  do {                                                                                     \
    ::pgb::count_launch();                                                                 \
    cudaError_t _e = cudaGetLastError();                                                   \
    if (_e != cudaSuccess) {                                                               \
      ::pgb::set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return PGB_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

// Character codes.  Nucleotides: "ACGTRYMKSWHBVDN-?X" (pplacer_src/nuc_models.ml:24-45);
// amino acids: "ARNDCQEGHILKMFPSTWYV" then B J Z X - ? (pplacer_src/prot_models.ml:5-43).
// '-' and '?' are the non-informative characters (common_src/alignment.ml:235).
constexpr int kNucCodes = 18;
constexpr int kAaCodes = 26;
constexpr int kMaxCodes = 26;
constexpr uint8_t kBadCode = 255;
inline const char *code_alphabet(int K) { return K == 4 ? "ACGTRYMKSWHBVDN-?X" : "ARNDCQEGHILKMFPSTWYVBJZX-?"; }
inline int n_codes(int K) { return K == 4 ? kNucCodes : kAaCodes; }
// likelihood vector of code c
void code_lv(int K, int c, double *lv);
inline bool code_informative(int K, int c) {
  return K == 4 ? (c != 15 && c != 16) : (c != 24 && c != 25);
}

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace pgb
