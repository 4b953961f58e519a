// common.cuh -- shared device/host helpers of libngia (internal header).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "ngia.h"

namespace ngia {

constexpr int kBands = NGIA_BANDS;
constexpr uint32_t kFull = 0xFFFFFFFFu;

// Records the CUDA error for ngia_last_cuda_error() and maps it to a status.
int cuda_fail(cudaError_t e);
#define NGIA_CUDA(call)                              \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return ::ngia::cuda_fail(e_); \
  } while (0)
// Every kernel launch site calls NGIA_LAUNCHED() right after its launch: it
// counts the launch (ngia_kernel_launches) and checks the launch error.
void note_launch();
// A captured graph's kernels: taken back after its capture (their launch
// sites counted them then), added at each replay.
void note_launches(long long delta);
#define NGIA_LAUNCHED()               \
  do {                                \
    ::ngia::note_launch();            \
    NGIA_CUDA(cudaGetLastError());    \
  } while (0)
#define NGIA_TRY(expr)          \
  do {                          \
    int s_ = (expr);            \
    if (s_ != NGIA_OK) return s_; \
  } while (0)

int round_mode();  // process-wide band-bound rounding (NGIA_ROUND_*)

inline cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

// ---- band geometry -----------------------------------------------------------
// The reference visits, for the 32-column block starting at residue i, the row
// blocks j in [max(i - lsft, 0), min(i + rsft, Lr)) with
//   lsft = (ceil(Lt - Lt*t) + 31) & ~31,  rsft = ceil(Lr - Lt*t) + 32
// (src/buildGraph.hpp:208-217).  In block units that is
//   J0(I) = max(I - ls, 0),  J1(I) = min(I + rs, nr)
// with ls = lsft/32, rs = ceil(rsft/32), nr = ceil(Lr/32): both ends advance by
// at most one block per column block, and at most min(ls + rs, nr) row blocks
// are live at once.
struct Band {
  uint32_t ls, rs, nr, nc;
  uint32_t width;  // max live row blocks = min(ls + rs, nr)
  bool pass;       // the length filter Lt >= Lr*t (src/buildGraph.hpp:201)
  uint32_t lr, lt;
  float t;
};

__host__ __device__ inline float identity_threshold(uint32_t identity) {
  return (float)identity / 100.0f;
}

// float -> uint32 of a ceil'd value; values <= 0 (and NaN) give 0, the GPU's
// saturating conversion.
__host__ __device__ inline uint32_t ceil_to_u32(float v) {
  float c = ceilf(v);
  return c > 0.0f ? (uint32_t)c : 0u;
}

__host__ __device__ inline Band make_band(uint32_t lr, uint32_t lt, float t,
                                          int fma_mode) {
  Band b;
  b.lr = lr;
  b.lt = lt;
  b.t = t;
  if (lr > NGIA_MAX_READ || lt > NGIA_MAX_READ) {
    // makedb never writes such records; refusing them keeps every row index
    // of the alignment inside its 2048-word bound.
    b.ls = b.rs = b.nr = b.nc = b.width = 0;
    b.pass = false;
    return b;
  }
#ifdef __CUDA_ARCH__
  const float flr = __uint2float_rn(lr), flt = __uint2float_rn(lt);
  b.pass = !(flt < __fmul_rn(flr, t));
  float dl, dr;
  if (fma_mode) {
    dl = __fmaf_rn(-flt, t, flt);
    dr = __fmaf_rn(-flt, t, flr);
  } else {
    const float p = __fmul_rn(flt, t);
    dl = __fsub_rn(flt, p);
    dr = __fsub_rn(flr, p);
  }
#else
  // Host: compiled with -ffp-contract=off, so each operation rounds here.
  const float flr = (float)lr, flt = (float)lt;
  b.pass = !(flt < flr * t);
  float dl, dr;
  if (fma_mode) {
    dl = std::fmaf(-flt, t, flt);
    dr = std::fmaf(-flt, t, flr);
  } else {
    const float p = flt * t;
    dl = flt - p;
    dr = flr - p;
  }
#endif
  const uint32_t lsft = (ceil_to_u32(dl) + 31u) & ~31u;
  const uint32_t rsft = ceil_to_u32(dr) + 32u;
  b.ls = lsft >> 5;
  b.rs = (rsft + 31u) >> 5;
  b.nr = (lr + 31u) >> 5;
  b.nc = (lt + 31u) >> 5;
  const uint32_t w = b.ls + b.rs;
  b.width = w < b.nr ? w : b.nr;
  return b;
}

// 32x32 blocks the reference loop visits for this pair:
//   sum over column blocks i < nc of max(0, min(i + rs, nr) - max(i - ls, 0)).
// Terms vanish from i = nr + ls on; below that both ends are arithmetic runs,
// so the sum has a closed form (checked against the loop on all small shapes).
__host__ __device__ inline uint64_t band_blocks(const Band &b) {
  if (!b.pass) return 0;
  const uint64_t ls = b.ls, rs = b.rs, nr = b.nr;
  const uint64_t nc = b.nc < nr + ls ? b.nc : nr + ls;  // columns with live rows
  const uint64_t up = nr > rs ? nr - rs : 0;            // columns with i + rs < nr
  const uint64_t a = nc < up ? nc : up;
  const uint64_t top = a * rs + a * (a - (a ? 1 : 0)) / 2 + (nc - a) * nr;
  const uint64_t m = nc > ls + 1 ? nc - 1 - ls : 0;
  return top - m * (m + 1) / 2;
}

// Final score from the LCS (src/buildGraph.hpp:245-252).
__host__ __device__ inline uint32_t identity_score(uint32_t lcs, uint32_t lr,
                                                   uint32_t lt, float t) {
  const uint32_t den = lr + lt - lcs;
#ifdef __CUDA_ARCH__
  const bool hit = __uint2float_rn(lcs) > __fmul_rn(__uint2float_rn(den), t);
#else
  const bool hit = (float)lcs > (float)den * t;
#endif
  return hit ? lcs * 100u / den : 0u;
}

// Early exit.  One column step raises the number of zero bits of the row
// vector (the running LCS) by at most one, and the score test
// lcs > (Lr + Lt - lcs) * t is monotone in lcs.  So once
//   lcs_so_far + columns_left
// fails the test, the pair's score is 0 whatever the remaining columns hold,
// and the alignment can stop: the score is exactly the reference's.
__host__ __device__ inline bool stream_may_reach(uint32_t lcs_so_far, uint32_t cols_done,
                                                 uint32_t lr, uint32_t lt, float t) {
  const uint32_t left = lt > cols_done ? lt - cols_done : 0u;
  uint32_t ub = lcs_so_far + left;
  const uint32_t cap = lr < lt ? lr : lt;
  if (ub > cap) ub = cap;
  return identity_score(ub, lr, lt, t) > 0;
}

// The same test for an upper bound of the final LCS itself.
__host__ __device__ inline bool lcs_may_reach(uint32_t ub, uint32_t lr, uint32_t lt, float t) {
  const uint32_t cap = lr < lt ? lr : lt;
  return identity_score(ub < cap ? ub : cap, lr, lt, t) > 0;
}

__host__ __device__ inline bool may_reach_threshold(uint32_t lcs_so_far, uint32_t cols_done,
                                                    const Band &b) {
  return stream_may_reach(lcs_so_far, cols_done, b.lr, b.lt, b.t);
}

template <typename T>
__host__ __device__ inline T ceil_div(T a, T b) {
  return (a + b - 1) / b;
}

}  // namespace ngia
