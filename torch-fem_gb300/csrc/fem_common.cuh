// Shared device/host helpers for the torch-fem GB300 kernels.
//
// Every entry point of the C-ABI (include/torchfem_gb300.h) returns an int
// status.  Device-side conditions (negative Jacobian, exceeded size limits,
// non-finite values) are OR-ed as bit flags into a caller-owned int32 status
// word, which the host reads after the stream has drained.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/torchfem_gb300.h"

namespace tfg {

// Device status bits (mirrors the FEM_* status codes: bit = 1 << code).
constexpr int kStatNonFinite = 1 << FEM_NONFINITE;
constexpr int kStatBadJacobian = 1 << FEM_BAD_JACOBIAN;
constexpr int kStatBounds = 1 << FEM_BOUNDS;

void set_last_error(const char* fmt, ...);

// Host-side count of kernel launches issued by this library (all threads).
void note_launch();

// Converts a pending CUDA error into FEM_CUDA_ERROR with a message.
int check_cuda(const char* where);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  return static_cast<unsigned int>(g);
}

__device__ __forceinline__ void flag_status(int32_t* status, int bits) {
  if (status) atomicOr(reinterpret_cast<int*>(status), bits);
}

// Warp-level sum (fixed butterfly order: deterministic).
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-level sum of a double; blockDim.x must be a multiple of 32 and
// <= 1024.  The result is valid in thread 0.  Fixed order: deterministic.
__device__ __forceinline__ double block_sum(double v, double* smem32) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) smem32[wid] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double t = (threadIdx.x < nw) ? smem32[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_sum(t);
  __syncthreads();
  return t;
}

// True in every thread of the CTA that arrives last at `counter` (one
// arrival per CTA); the caller resets the counter.
__device__ __forceinline__ bool arrive_last(unsigned int* counter) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

// Sum of partial[0..n)*stride+k in a fixed order (single CTA).
__device__ __forceinline__ double sum_partials(const double* partial, int n, int stride, int k,
                                               double* red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(partial + (int64_t)i * stride + k);
  return block_sum(s, red);
}

// L2 eviction-priority hints (PTX createpolicy / ld.L2::cache_hint): the part
// of the matrix that should stay resident in L2 across CG iterations is read
// evict_last, the streamed remainder evict_first.
__device__ __forceinline__ uint64_t l2_policy(bool keep) {
  uint64_t pol;
  if (keep) asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  else asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ float ld_l2(const float* ptr, uint64_t pol) {
  float v;
  asm("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(ptr), "l"(pol));
  return v;
}

__device__ __forceinline__ double ld_l2(const double* ptr, uint64_t pol) {
  double v;
  asm("ld.global.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(ptr), "l"(pol));
  return v;
}

__device__ __forceinline__ int32_t ld_l2(const int32_t* ptr, uint64_t pol) {
  int32_t v;
  asm("ld.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(ptr), "l"(pol));
  return v;
}

// Mixed precision keeps the residual it iterates on near unit norm: the FP32
// vectors hold r * rscale with rscale a power of two (exact to apply and to
// undo), so their dot products stay far from FP32 underflow and overflow at
// any problem scale and any depth of refinement.
__device__ __forceinline__ double unit_scale(double norm2) {
  if (!(norm2 > 0.0) || !isfinite(norm2)) return 1.0;
  int e;
  frexp(norm2, &e);
  return ldexp(1.0, -(e / 2));
}

}  // namespace tfg

#define TFG_CHECK_LAUNCH(where)                      \
  do {                                               \
    int _rc = ::tfg::check_cuda(where);              \
    if (_rc != FEM_OK) return _rc;                   \
  } while (0)

// Element-type dispatch: TFG_BODY runs with NE (nodes), D (dimension) and
// NIP (integration points) as compile-time constants.
#define TFG_ETYPE_CASE(ID, NE_, D_, NIP_) \
  case ID: {                              \
    constexpr int NE = NE_;               \
    constexpr int D = D_;                 \
    constexpr int NIP = NIP_;             \
    TFG_BODY;                             \
  } break;

#define TFG_DISPATCH_ETYPE(etype)                        \
  switch (etype) {                                       \
    TFG_ETYPE_CASE(FEM_QUAD1, 4, 2, 4)                   \
    TFG_ETYPE_CASE(FEM_HEXA1, 8, 3, 8)                   \
    TFG_ETYPE_CASE(FEM_TETRA2, 10, 3, 4)                 \
    TFG_ETYPE_CASE(FEM_TETRA1, 4, 3, 1)                  \
    TFG_ETYPE_CASE(FEM_TRIA1, 3, 2, 1)                   \
    TFG_ETYPE_CASE(FEM_QUAD2, 8, 2, 4)                   \
    TFG_ETYPE_CASE(FEM_TRIA2, 6, 2, 3)                   \
    TFG_ETYPE_CASE(FEM_HEXA2, 20, 3, 8)                  \
    default:                                             \
      set_last_error("unsupported element type %d", etype); \
      return FEM_INVALID;                                \
  }

