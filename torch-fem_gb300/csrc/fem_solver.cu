// Assembly (FEM.assemble_matrix, src/torchfem/base.py:398-426), Jacobi and
// block-Jacobi preconditioners, and the preconditioned CG solvers that replace
// the sparse_solve backends (src/torchfem/sparse.py:271-514).
//
// Determinism: every sum runs in a fixed order.  Assembly sums a slot's
// contributions in ascending element order from +0.0 (the order CPU
// index_add_ visits them), and all CG reductions are two-stage: per-CTA
// partials in a fixed tree, then a fixed-order sum by whichever CTA arrives
// last.  No floating-point atomics are used anywhere.
#include <algorithm>
#include <mutex>
#include <vector>

#include "fem_common.cuh"

namespace tfg {

int etype_info(int etype, int* ne, int* d, int* nip);
size_t scan_workspace_bytes(int64_t n);
int scan_exclusive(const int64_t* in, int64_t* out, int64_t n, int64_t* ws, cudaStream_t st);


// ---------------------------------------------------------------- assembly --
// Thread per node-pair block (a, b): gathers the d x d sub-blocks of every
// contributing element matrix, sums them in ascending element order and
// writes them with the Dirichlet condensation of base.py:414-419.
// Position of component c of block slot k of row a in the sliced layout:
// slices of 32 rows, slot-major, each component contiguous over the 32 rows.
__device__ __forceinline__ int64_t sell_index(const int64_t* __restrict__ sell_base, int64_t a, int64_t k,
                                              int c, int DD) {
  const int64_t s = a >> 5;
  const int lane = (int)(a & 31);
  return sell_base[s] * DD + (k * DD + c) * 32 + lane;
}

template <typename KT, typename AT, bool kSELL, int MAXD = 3>
__global__ void k_assemble(int n_e, int D, int64_t n_blocks, const int64_t* __restrict__ nbr_ptr,
                           const int32_t* __restrict__ nbr, const int64_t* __restrict__ blk_ptr,
                           const int32_t* __restrict__ contrib, const int32_t* __restrict__ blk_row,
                           const int64_t* __restrict__ inc_ptr, const KT* __restrict__ ke,
                           const int64_t* __restrict__ row_ptr, const uint8_t* __restrict__ con,
                           double* __restrict__ val, const int64_t* __restrict__ sell_base,
                           float* __restrict__ sval, double* __restrict__ sval64 = nullptr) {
  const int64_t blk = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (blk >= n_blocks) return;
  const int64_t a = blk_row[blk];
  const int64_t b = nbr[blk];
  const int64_t k = blk - nbr_ptr[a];
  const int ND = n_e * D;
  const int nn = n_e * n_e;
  AT acc[MAXD][MAXD];
#pragma unroll
  for (int i = 0; i < MAXD; ++i)
#pragma unroll
    for (int j = 0; j < MAXD; ++j) acc[i][j] = AT(0);
  for (int64_t q = blk_ptr[blk]; q < blk_ptr[blk + 1]; ++q) {
    const int32_t c = contrib[q];
    const int64_t e = c / nn;
    const int la = (c / n_e) % n_e, lb = c % n_e;
    const KT* src = ke + e * (int64_t)ND * ND + (int64_t)(la * D) * ND + lb * D;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) acc[i][j] += (AT)src[i * ND + j];
  }
  const bool orphan = inc_ptr[a + 1] == inc_ptr[a];
  for (int i = 0; i < D; ++i) {
    const int64_t r = a * D + i;
    const bool rc = con[r] != 0;
    for (int j = 0; j < D; ++j) {
      const int64_t cdof = b * D + j;
      double v = (double)acc[i][j];
      if (rc || con[cdof]) v = 0.0;
      if (r == cdof && rc) v = 1.0;
      if (kSELL) {
        const int64_t at = sell_index(sell_base, a, k, i * D + j, D * D);
        sval[at] = (float)v;
        if (sval64) sval64[at] = v;
      } else {
        if (orphan) {
          if (i == j) val[row_ptr[r]] = v;
        } else {
          val[row_ptr[r] + k * D + j] = v;
        }
      }
    }
  }
}

// FP64 y = A x over the FP64 copy of the sliced matrix (fem_assemble_sell_pair):
// the mixed solvers' residual replacement.  The copy is the condensed matrix
// itself (identity rows and columns at constrained DOFs), so y equals the
// element pass with constrained entries zeroed and y = x there.  Blocks of
// 2x2 / 3x3: one slice per CTA, kApplyW warps sharing its slots, partial rows
// summed in shared memory in a fixed order; scalar rows: a warp per slice,
// a thread per row, four slots' loads in flight.  Bound by the FP64 pipe
// (one FMA per stored value) more than by the 8-byte values.
constexpr int kApplyW = 4;

template <int D>
__global__ void __launch_bounds__(kApplyW * 32) k_sell_apply64(int64_t n_rows, int64_t n_slices,
                                                               const int64_t* __restrict__ sell_base,
                                                               const int32_t* __restrict__ col,
                                                               const double* __restrict__ sval,
                                                               const double* __restrict__ x,
                                                               double* __restrict__ y) {
  constexpr int DD = D * D;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t pol = l2_policy(false);
  if constexpr (D == 1) {
    const int64_t s = (int64_t)blockIdx.x * kApplyW + w;
    if (s >= n_slices) return;
    const int64_t b0 = sell_base[s];
    const int len = (int)((sell_base[s + 1] - b0) >> 5);
    const int32_t* cp = col + b0 + lane;
    const double* vp = sval + b0 + lane;
    double acc = 0.0;
    int k = 0;
    for (; k + 4 <= len; k += 4) {
      int32_t cc[4];
      double mv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        cc[u] = ld_l2(cp + (int64_t)(k + u) * 32, pol);
        mv[u] = ld_l2(vp + (int64_t)(k + u) * 32, pol);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) acc = fma(mv[u], x[cc[u]], acc);
    }
    for (; k < len; ++k) acc = fma(ld_l2(vp + (int64_t)k * 32, pol), x[ld_l2(cp + (int64_t)k * 32, pol)], acc);
    const int64_t i = s * 32 + lane;
    if (i < n_rows) y[i] = acc;
  } else {
    __shared__ double ys[kApplyW][D][32];
    const int64_t s = blockIdx.x;
    const int64_t b0 = sell_base[s];
    const int len = (int)((sell_base[s + 1] - b0) >> 5);
    const int32_t* cp = col + b0 + lane;
    const double* vp = sval + b0 * DD + lane;
    double acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = 0.0;
#pragma unroll 2
    for (int k = w; k < len; k += kApplyW) {
      const int64_t cc = ld_l2(cp + (int64_t)k * 32, pol);
      const double* vk = vp + (int64_t)k * DD * 32;
      double m[DD];
#pragma unroll
      for (int e = 0; e < DD; ++e) m[e] = ld_l2(vk + e * 32, pol);
      double xv[D];
#pragma unroll
      for (int j = 0; j < D; ++j) xv[j] = x[cc * D + j];
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int j = 0; j < D; ++j) acc[r] = fma(m[r * D + j], xv[j], acc[r]);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) ys[w][c][lane] = acc[c];
    __syncthreads();
    if (w == 0) {
      const int64_t i = s * 32 + lane;
      if (i < n_rows) {
#pragma unroll
        for (int c = 0; c < D; ++c) {
          double t = ys[0][c][lane];
#pragma unroll
          for (int u = 1; u < kApplyW; ++u) t += ys[u][c][lane];
          y[i * D + c] = t;
        }
      }
    }
  }
}

__global__ void k_jacobi(const double* __restrict__ val, const int64_t* __restrict__ diag_map, int64_t n,
                         double* __restrict__ inv, int32_t* status) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double d = val[diag_map[r]];
  const double v = 1.0 / d;
  if (!isfinite(v)) flag_status(status, kStatNonFinite);
  inv[r] = v;
}

__global__ void k_block_jacobi(const float* __restrict__ sval, const int64_t* __restrict__ sell_base,
                               const int64_t* __restrict__ nbr_ptr, const int64_t* __restrict__ diag_blk,
                               int64_t n_nod, int D, float* __restrict__ inv, int32_t* status) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nod) return;
  const int64_t k = diag_blk[a] - nbr_ptr[a];
  double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) M[i][j] = sval[sell_index(sell_base, a, k, i * D + j, D * D)];
  double R[3][3];
  double det;
  if (D == 2) {
    det = M[0][0] * M[1][1] - M[0][1] * M[1][0];
    R[0][0] = M[1][1] / det;
    R[0][1] = -M[0][1] / det;
    R[1][0] = -M[1][0] / det;
    R[1][1] = M[0][0] / det;
  } else if (D == 3) {
    const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    const double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    const double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
    R[0][0] = c00 / det;
    R[1][0] = c01 / det;
    R[2][0] = c02 / det;
    R[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
    R[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
    R[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
    R[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
    R[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
    R[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
  } else {
    det = M[0][0];
    R[0][0] = 1.0 / det;
  }
  bool ok = isfinite(det) && det != 0.0;
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) {
      inv[a * D * D + i * D + j] = (float)R[i][j];
      ok = ok && isfinite(R[i][j]);
    }
  if (!ok) flag_status(status, kStatNonFinite);
}

// --------------------------------------------------------------------- CG ---
enum {
  kDoneNo = 0,
  kDoneConverged = 1,
  kDoneMaxIter = 2,
  kDoneNonFinite = 3,
  kDoneBreakdown = 4,
  kDoneBarrierTimeout = 5
};

struct Ctrl {
  double rz;       // r.z of the current iterate
  double rz_new;   // r.z after the last update (held while a replacement is pending)
  double alpha;
  double beta;
  double rr;       // ||r||^2 of the working residual
  double rr_ref;   // ||r||^2 at the last FP64 replacement (mixed)
  double rr_true;  // ||b - A x||^2 from the last FP64 replacement (mixed)
  double bb;       // ||b||^2
  double tol2bb;   // rtol^2 ||b||^2
  double rscale;   // power of two applied to the residual held by the CG vectors (mixed; 1 for FP64)
  double tol2_lo;  // tol2bb in the units of the CG vectors (tol2bb * rscale^2)
  double delta2;   // replacement threshold (mixed)
  long long iters;
  long long max_iter;
  long long replacements;
  int done;
  int replace;
  int mixed;
  unsigned int counter;
  int bar_error;             // persistent kernel: a barrier wait ran out
  unsigned long long bar_seq;  // persistent kernel: grid-barrier arrivals, never reset within a solve
};

// Two block sums in one pass (fixed order).  Valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b, double2* smem32) {
  a = warp_sum(a);
  b = warp_sum(b);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) smem32[wid] = make_double2(a, b);
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double2 t = (threadIdx.x < nw) ? smem32[threadIdx.x] : make_double2(0.0, 0.0);
  if (wid == 0) {
    t.x = warp_sum(t.x);
    t.y = warp_sum(t.y);
  }
  a = t.x;
  b = t.y;
  __syncthreads();
}

__device__ __forceinline__ bool ctrl_idle(const Ctrl* c) {
  return (*(volatile const int*)&c->done) != 0 || (*(volatile const int*)&c->replace) != 0;
}

// Scalar CSR FP64 SpMV q = A p with TPR threads per row, fused p.q partial;
// the last CTA forms alpha = rz / p.q.
template <int TPR>
__global__ void __launch_bounds__(256)
k_spmv_csr(int64_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
           const double* __restrict__ val, const double* __restrict__ p, double* __restrict__ q,
           double* __restrict__ partial, Ctrl* ctrl, int64_t keep_nnz) {
  __shared__ double red[32];
  if (ctrl_idle(ctrl)) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = t / TPR;
  const int sub = (int)(t % TPR);
  double pq = 0.0;
  double s = 0.0;
  if (row < n) {
    const int64_t rs = row_ptr[row], re = row_ptr[row + 1];
    const uint64_t pol = l2_policy(rs < keep_nnz);
    for (int64_t j = rs + sub; j < re; j += TPR) s += ld_l2(val + j, pol) * p[ld_l2(col + j, pol)];
  }
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
  if (row < n && sub == 0) {
    q[row] = s;
    pq = p[row] * s;
  }
  const double bsum = block_sum(pq, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = bsum;
  if (arrive_last(&ctrl->counter)) {
    const double tot = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      if (tot == 0.0 || !isfinite(tot)) {
        ctrl->done = isfinite(tot) ? kDoneBreakdown : kDoneNonFinite;
      } else {
        ctrl->alpha = ctrl->rz / tot;
      }
    }
  }
}

// Sliced block SpMV, FP32: thread per node row, slices of 32 rows stored
// slot-major with every block component contiguous over the slice, so each
// load instruction of a warp reads one full 128-byte line.  FP32 products and
// accumulation; the p.q partial is formed in FP64.
constexpr int kSellWarps = 4;  // warps sharing one slice's slots

template <int D>
__global__ void __launch_bounds__(kSellWarps * 32)
k_spmv_sell(int64_t n_rows, const int64_t* __restrict__ sell_base, const int32_t* __restrict__ col,
            const float* __restrict__ sval, const float* __restrict__ p, float* __restrict__ q,
            double* __restrict__ partial, Ctrl* ctrl, int64_t keep_slots) {
  constexpr int DD = D * D;
  __shared__ float ys[kSellWarps][D][32];
  __shared__ double red[32];
  if (ctrl_idle(ctrl)) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t n_slices = (n_rows + 31) >> 5;
  double pq = 0.0;
  for (int64_t s = blockIdx.x; s < n_slices; s += gridDim.x) {
    const int64_t b0 = sell_base[s];
    const int len = (int)((sell_base[s + 1] - b0) >> 5);
    const uint64_t pol = l2_policy(b0 < keep_slots);
    const int32_t* cp = col + b0 + lane;
    const float* vp = sval + b0 * DD + lane;
    float y[D];
#pragma unroll
    for (int i = 0; i < D; ++i) y[i] = 0.f;
#pragma unroll 2
    for (int k = w; k < len; k += kSellWarps) {
      const int64_t c = ld_l2(cp + (int64_t)k * 32, pol);
      const float* vk = vp + (int64_t)k * DD * 32;
      float m[DD];
#pragma unroll
      for (int e = 0; e < DD; ++e) m[e] = ld_l2(vk + e * 32, pol);
      float x[D];
#pragma unroll
      for (int j = 0; j < D; ++j) x[j] = p[c * D + j];
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) y[i] = fmaf(m[i * D + j], x[j], y[i]);
    }
#pragma unroll
    for (int i = 0; i < D; ++i) ys[w][i][lane] = y[i];
    __syncthreads();
    if (w == 0) {
      const int64_t a = s * 32 + lane;
      if (a < n_rows) {
#pragma unroll
        for (int i = 0; i < D; ++i) {
          float t = ys[0][i][lane];
#pragma unroll
          for (int v = 1; v < kSellWarps; ++v) t += ys[v][i][lane];
          q[a * D + i] = t;
          pq += (double)p[a * D + i] * (double)t;
        }
      }
    }
    __syncthreads();
  }
  const double bsum = block_sum(pq, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = bsum;
  if (arrive_last(&ctrl->counter)) {
    const double tot = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      if (tot == 0.0 || !isfinite(tot)) {
        ctrl->done = isfinite(tot) ? kDoneBreakdown : kDoneNonFinite;
      } else {
        ctrl->alpha = ctrl->rz / tot;
      }
    }
  }
}

// Slice lengths: 32 x (largest degree among the slice's rows).
__global__ void k_sell_len(const int64_t* __restrict__ nbr_ptr, int64_t n_nod, int64_t* __restrict__ len) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n_slices = (n_nod + 31) >> 5;
  if (s >= n_slices) return;
  int64_t m = 0;
  for (int l = 0; l < 32; ++l) {
    const int64_t a = s * 32 + l;
    if (a < n_nod) m = max(m, nbr_ptr[a + 1] - nbr_ptr[a]);
  }
  len[s] = 32 * m;
}

// Column of every slot; padding slots point at the row itself (value 0).
__global__ void k_sell_cols(const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                            int64_t n_nod, const int64_t* __restrict__ sell_base, int32_t* __restrict__ col) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n_slices = (n_nod + 31) >> 5;
  if (a >= n_slices * 32) return;
  const int64_t s = a >> 5;
  const int lane = (int)(a & 31);
  const int64_t b0 = sell_base[s];
  const int64_t len = (sell_base[s + 1] - b0) >> 5;
  const int64_t deg = a < n_nod ? nbr_ptr[a + 1] - nbr_ptr[a] : 0;
  const int32_t pad = a < n_nod ? (int32_t)a : 0;
  for (int64_t k = 0; k < len; ++k) col[b0 + k * 32 + lane] = k < deg ? nbr[nbr_ptr[a] + k] : pad;
}

// z = M r for one group of G DOFs: Jacobi (G = 1, FP64 inverse diagonal) or
// block Jacobi (G = dim, FP32 inverse blocks).
template <int G, typename VT>
__device__ __forceinline__ void apply_prec(const void* prec, int64_t i, const VT (&r)[G], VT (&z)[G]) {
  if constexpr (G == 1) {
    z[0] = (VT)(((const double*)prec)[i] * (double)r[0]);
  } else {
    const float* m = (const float*)prec + i * G * G;
#pragma unroll
    for (int a = 0; a < G; ++a) {
      float s = 0.f;
#pragma unroll
      for (int b = 0; b < G; ++b) s = fmaf(m[a * G + b], (float)r[b], s);
      z[a] = (VT)s;
    }
  }
}

// Finalisation shared by the update and replacement kernels.
__device__ void finish_update(Ctrl* c, double rz_new, double rr, bool count_iter) {
  if (count_iter) c->iters += 1;
  c->rr = rr;
  if (!isfinite(rr) || !isfinite(rz_new)) {
    c->done = kDoneNonFinite;
    return;
  }
  bool stop = false;
  if (c->mixed) {
    if (rr <= c->tol2_lo || rr <= c->delta2 * c->rr_ref) {
      c->replace = 1;
      c->rz_new = rz_new;
      stop = true;
    }
  } else if (rr <= c->tol2_lo) {
    c->done = kDoneConverged;
    stop = true;
  }
  if (!stop && c->iters >= c->max_iter) {
    c->done = kDoneMaxIter;
    c->rz_new = rz_new;
    return;
  }
  if (!stop) {
    c->beta = rz_new / c->rz;
    c->rz = rz_new;
  }
}

// x += alpha p; r -= alpha q; z = M r; partial r.z and r.r.  Grid-stride
// over groups of G DOFs (a node for block Jacobi).
template <int G, typename VT>
__global__ void __launch_bounds__(256)
k_update(int64_t n_groups, VT* __restrict__ x, VT* __restrict__ r, const VT* __restrict__ p,
         const VT* __restrict__ q, VT* __restrict__ z, const void* __restrict__ prec,
         double* __restrict__ partial, Ctrl* ctrl) {
  __shared__ double2 red2[32];
  __shared__ double red[32];
  if (ctrl_idle(ctrl)) return;
  double rz = 0.0, rr = 0.0;
  const VT alpha = (VT)ctrl->alpha;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_groups;
       i += (int64_t)gridDim.x * blockDim.x) {
    VT rv[G], zv[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int64_t k = i * G + g;
      x[k] += alpha * p[k];
      rv[g] = r[k] - alpha * q[k];
      r[k] = rv[g];
    }
    apply_prec<G, VT>(prec, i, rv, zv);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      z[i * G + g] = zv[g];
      rz += (double)rv[g] * (double)zv[g];
      rr += (double)rv[g] * (double)rv[g];
    }
  }
  block_sum2(rz, rr, red2);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = rz;
    partial[2 * blockIdx.x + 1] = rr;
  }
  if (arrive_last(&ctrl->counter)) {
    const double t1 = sum_partials(partial, gridDim.x, 2, 0, red);
    const double t2 = sum_partials(partial, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      finish_update(ctrl, t1, t2, true);
    }
  }
}

template <typename VT>
__global__ void __launch_bounds__(256) k_pupdate(int64_t n, const VT* __restrict__ z, VT* __restrict__ p, Ctrl* ctrl) {
  if (ctrl_idle(ctrl)) return;
  const VT beta = (VT)ctrl->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// Start (x = 0): r = b * rscale, z = M r, p = z; rz, rr, bb; tolerances.
template <int G, typename VT>
__global__ void __launch_bounds__(256)
k_init(int64_t n_groups, const double* __restrict__ b, VT* __restrict__ x, VT* __restrict__ r,
       VT* __restrict__ z, VT* __restrict__ p, const void* __restrict__ prec,
       double* __restrict__ partial, Ctrl* ctrl, double rtol2) {
  __shared__ double red[32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double sc = ctrl->rscale;
  double rz = 0.0, rr = 0.0, bb = 0.0;
  if (i < n_groups) {
    VT rv[G], zv[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const double bv = b[i * G + g];
      bb += bv * bv;
      rv[g] = (VT)(bv * sc);
      r[i * G + g] = rv[g];
      x[i * G + g] = VT(0);
    }
    apply_prec<G, VT>(prec, i, rv, zv);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      z[i * G + g] = zv[g];
      p[i * G + g] = zv[g];
      rz += (double)rv[g] * (double)zv[g];
      rr += (double)rv[g] * (double)rv[g];
    }
  }
  const double s1 = block_sum(rz, red);
  const double s2 = block_sum(rr, red);
  const double s3 = block_sum(bb, red);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = s1;
    partial[3 * blockIdx.x + 1] = s2;
    partial[3 * blockIdx.x + 2] = s3;
  }
  if (arrive_last(&ctrl->counter)) {
    const double t1 = sum_partials(partial, gridDim.x, 3, 0, red);
    const double t2 = sum_partials(partial, gridDim.x, 3, 1, red);
    const double t3 = sum_partials(partial, gridDim.x, 3, 2, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      ctrl->rz = t1;
      ctrl->rr = t2;
      ctrl->rr_ref = t2;
      ctrl->rr_true = t3;
      ctrl->bb = t3;
      ctrl->tol2bb = rtol2 * t3;
      ctrl->tol2_lo = ctrl->tol2bb * sc * sc;
      ctrl->iters = 0;
      ctrl->replacements = 0;
      ctrl->replace = 0;
      if (!isfinite(t1) || !isfinite(t3)) ctrl->done = kDoneNonFinite;
      else if (t3 == 0.0 || t2 <= ctrl->tol2_lo) ctrl->done = kDoneConverged;
      else ctrl->done = kDoneNo;
    }
  }
}

// Mixed precision start: ||b||^2 and the first residual scale.
__global__ void __launch_bounds__(256) k_bnorm(int64_t n, const double* __restrict__ b,
                                               double* __restrict__ partial, Ctrl* ctrl) {
  __shared__ double red[32];
  double t = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    t += b[i] * b[i];
  t = block_sum(t, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (arrive_last(&ctrl->counter)) {
    const double bb = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      ctrl->rscale = unit_scale(bb);
    }
  }
}

// Mixed precision: fold the FP32 correction (in residual-scale units) into
// the FP64 solution.
__global__ void k_fold(int64_t n, double* __restrict__ x64, float* __restrict__ xlo, const Ctrl* ctrl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double inv = 1.0 / ctrl->rscale;  // a power of two: exact
  x64[i] += (double)xlo[i] * inv;
  xlo[i] = 0.f;
}

// Mixed precision replacement: r = b - y (FP64), r_lo = (float)(r * s) with s
// the unit scale of the previous true residual, z = M r_lo, new r.z / r.r;
// the kept direction p is rescaled through beta.  Convergence is decided on
// the FP64 residual.
template <int G>
__global__ void __launch_bounds__(256)
k_replace(int64_t n_groups, const double* __restrict__ b, const double* __restrict__ y,
          float* __restrict__ rlo, float* __restrict__ z, const void* __restrict__ prec,
          double* __restrict__ partial, Ctrl* ctrl) {
  __shared__ double red[32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double sc_old = ctrl->rscale;
  const double sc = unit_scale(ctrl->rr_true);
  double rz = 0.0, rr = 0.0, r64 = 0.0;
  if (i < n_groups) {
    float rv[G], zv[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int64_t k = i * G + g;
      const double rd = b[k] - y[k];
      r64 += rd * rd;
      rv[g] = (float)(rd * sc);
      rlo[k] = rv[g];
    }
    apply_prec<G, float>(prec, i, rv, zv);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      z[i * G + g] = zv[g];
      rz += (double)rv[g] * (double)zv[g];
      rr += (double)rv[g] * (double)rv[g];
    }
  }
  const double s1 = block_sum(rz, red);
  const double s2 = block_sum(rr, red);
  const double s3 = block_sum(r64, red);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = s1;
    partial[3 * blockIdx.x + 1] = s2;
    partial[3 * blockIdx.x + 2] = s3;
  }
  if (arrive_last(&ctrl->counter)) {
    const double t1 = sum_partials(partial, gridDim.x, 3, 0, red);
    const double t2 = sum_partials(partial, gridDim.x, 3, 1, red);
    const double t3 = sum_partials(partial, gridDim.x, 3, 2, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      ctrl->rr_true = t3;
      ctrl->replacements += 1;
      ctrl->replace = 0;
      if (!isfinite(t3) || !isfinite(t1)) {
        ctrl->done = kDoneNonFinite;
      } else if (t3 <= ctrl->tol2bb) {
        ctrl->done = kDoneConverged;
      } else if (ctrl->done == kDoneNo) {
        // p_old holds the old scale: p = z + beta * p with beta = (t1 / rz) / f
        // (f = sc / sc_old) continues the same direction in the new scale
        ctrl->rr = t2;
        ctrl->rr_ref = t2;
        ctrl->beta = t1 / ctrl->rz * (sc_old / sc);
        ctrl->rz = t1;
        ctrl->rscale = sc;
        ctrl->tol2_lo = ctrl->tol2bb * sc * sc;
      }
    }
  }
}

// FP32 solution (in residual-scale units) to FP64.
__global__ void k_copy_cast(int64_t n, const float* __restrict__ in, double* __restrict__ out, const Ctrl* ctrl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i] * (1.0 / ctrl->rscale);
}


// ------------------------------------------------------- persistent CG ------
// One cooperative launch runs CG iterations until convergence, a pending FP64
// replacement (mixed) or the iteration cap.  Each CTA owns a contiguous range
// of rows (slices for the sliced layout): it computes q = A p for them, then
// updates x, r, z and p for the same rows, so the only data crossing CTAs are
// the gathered p values and three scalars per iteration.  Three grid barriers
// per iteration; every CTA sums the per-CTA partials itself in one fixed
// order, so all CTAs take identical decisions and results are deterministic.
// The matrix is streamed with L2 evict_first; the CG vectors stay in L2.
constexpr int kCsrTpr = 8;  // lanes per scalar CSR row
// CSR rows longer than kLongRow entries (a reference point's rows in a coupled
// system hold every DOF next to its coupled face) are reduced by the whole CTA
// after the short rows, in one fixed order; a group of kCsrTpr lanes would take
// one row that long serially while every other CTA waits at the next barrier.
// A CTA lists its first kLongMax long rows at launch; later ones stay with the
// lane groups.
constexpr int kLongRow = 512;
constexpr int kLongMax = 32;
#ifndef TFG_PTHREADS
#define TFG_PTHREADS 512
#endif
constexpr int kPThreads = TFG_PTHREADS;
constexpr int kPKS = 4;  // warps sharing one slice (sliced layout)

struct PersistParams {
  int64_t n;
  int64_t n_rows;
  const int64_t* row_ptr;  // CSR row pointers or sell_base
  const int32_t* col;
  const void* val;
  const void* prec;
  void* x;
  void* r;
  void* z;
  void* p;
  void* q;
  double* partial;  // [3 * gridDim.x]
  Ctrl* ctrl;
  long long spin_limit;  // clock cycles a barrier wait may last
};

// Grid barrier with a bounded wait, fused with the fixed-order sum of NK
// per-CTA partials.  One monotonic 64-bit arrival counter: every CTA adds 1
// (release) and polls (relaxed, with a short sleep, so that polling neither
// floods the counter's L2 slice nor invalidates L1 lines a co-resident CTA is
// using) until the count reaches the next multiple of the grid size; one
// acquire fence follows.  No reset step sits on the critical path: the counter
// starts at 0 for each solve and every launch passes whole barriers only.
// Then warp 0 alone sums partial[3*i + k0 + j] over the CTAs i in one fixed
// order and shares the sums through shared memory, so every thread of every
// CTA holds identical values.  Returns false (on every thread) once any CTA's
// wait has run out; the kernel then stops.
template <int NK, typename F>
__device__ __forceinline__ bool grid_barrier(Ctrl* c, long long spin_limit, const double* partial, int k0, F&& on_sums) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x < 32) {
    if (threadIdx.x == 0) {
      unsigned long long old;
      asm volatile("atom.add.release.gpu.u64 %0, [%1], 1;" : "=l"(old) : "l"(&c->bar_seq) : "memory");
      const unsigned long long target = (old / gridDim.x + 1) * gridDim.x;
      const long long t0 = clock64();
      while (true) {
        unsigned long long now;
        asm volatile("ld.relaxed.gpu.u64 %0, [%1];" : "=l"(now) : "l"(&c->bar_seq) : "memory");
        if (now >= target) break;
        if (*(volatile int*)&c->bar_error) break;
        if (clock64() - t0 > spin_limit) {
          atomicExch(&c->bar_error, 1);
          break;
        }
        __nanosleep(32);
      }
      asm volatile("fence.acq_rel.gpu;" ::: "memory");
      ok = (*(volatile int*)&c->bar_error) == 0;
    }
    __syncwarp();
    if constexpr (NK > 0) {
      const int lane = threadIdx.x;
      double sums[NK];
#pragma unroll
      for (int j = 0; j < NK; ++j) {
        double v = 0.0;
        for (int i = lane; i < (int)gridDim.x; i += 32) v += __ldcg(partial + 3 * i + k0 + j);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        sums[j] = v;
      }
      if (lane == 0) on_sums(sums);
    }
  }
  __syncthreads();
  return ok != 0;
}

// Fixed-order CTA sum of N per-thread accumulators: shuffle tree within each
// warp, then thread 0 adds the warp sums in FP64 and stores them to out[j].
template <int N, typename ACC>
__device__ __forceinline__ void cta_partials(ACC (&v)[N], double* out, double (*wsum)[2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < N; ++j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[j].shfl_down(o);
  }
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) wsum[warp][j] = v[j].value();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w][j];
      out[j] = t;
    }
  }
}

// Dot-product accumulators of the persistent CG.  On the FP32 (mixed) path a
// float-float pair: each product is split exactly (a*b and its FMA residual)
// and summed with Knuth's TwoSum, which keeps the sums as accurate as FP64
// accumulation of the FP32 products while running on the FP32 pipe (the FP64
// pipe of this GPU is a small fraction of the FP32 rate).  On the FP64 path a
// plain double.
template <typename VT> struct DotAcc;
template <> struct DotAcc<double> {
  double v = 0.0;
  __device__ __forceinline__ void fma(double a, double b) { v = ::fma(a, b, v); }
  __device__ __forceinline__ void shfl_down(int o) { v += __shfl_down_sync(0xffffffffu, v, o); }
  __device__ __forceinline__ double value() const { return v; }
};
// (round-to-nearest intrinsics: never contracted into an FMA)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
template <> struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x, float x_lo) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, x_lo));
  }
  __device__ __forceinline__ void fma(float a, float b) {
    const float p = __fmul_rn(a, b);
    add(p, fmaf(a, b, -p));
  }
  __device__ __forceinline__ void shfl_down(int o) {
    const float h = __shfl_down_sync(0xffffffffu, hi, o);
    const float l = __shfl_down_sync(0xffffffffu, lo, o);
    add(h, l);
    const float t = __fadd_rn(hi, lo);  // renormalise
    lo = __fsub_rn(lo, __fsub_rn(t, hi));
    hi = t;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// First i in [0, n] with base[i] >= target (base non-decreasing).
__device__ __forceinline__ int64_t lower_bound_i64(const int64_t* base, int64_t n, int64_t target) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (base[mid] < target) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <typename VT> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int W = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int W = 2; };

template <typename V, typename T>
__device__ __forceinline__ T& lane_of(V& v, int i) { return reinterpret_cast<T*>(&v)[i]; }

// p[k] = z[k] + beta p[k] for k in [lo, hi): 16-byte vectors over the aligned
// middle, U per thread in flight, scalar head and tail.
template <typename VT, int U>
__device__ __forceinline__ void direction_update(VT* __restrict__ p, const VT* __restrict__ z, VT beta,
                                                 int64_t lo, int64_t hi) {
  using V = typename Vec16<VT>::type;
  constexpr int W = Vec16<VT>::W;
  const int64_t a = min(hi, (lo + W - 1) / W * W);
  const int64_t b = max(a, hi / W * W);
  for (int64_t k = lo + threadIdx.x; k < a; k += blockDim.x) p[k] = z[k] + beta * p[k];
  for (int64_t k = b + threadIdx.x; k < hi; k += blockDim.x) p[k] = z[k] + beta * p[k];
  V* pv = reinterpret_cast<V*>(p + a);
  const V* zv = reinterpret_cast<const V*>(z + a);
  const int64_t nv = (b - a) / W;
  for (int64_t i0 = threadIdx.x; i0 < nv; i0 += U * (int64_t)blockDim.x) {
    V pp[U], zz[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + (int64_t)u * blockDim.x;
      if (i < nv) {
        pp[u] = pv[i];
        zz[u] = zv[i];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + (int64_t)u * blockDim.x;
      if (i < nv) {
#pragma unroll
        for (int w = 0; w < W; ++w) lane_of<V, VT>(pp[u], w) = lane_of<V, VT>(zz[u], w) + beta * lane_of<V, VT>(pp[u], w);
        pv[i] = pp[u];
      }
    }
  }
}

// One node of the solution/residual update: x += alpha p, r -= alpha q,
// z = M r; accumulates r.z and r.r.
template <int G, typename VT>
__device__ __forceinline__ void node_update(const void* prec, int64_t a, VT alpha, VT* __restrict__ x,
                                            VT* __restrict__ r, VT* __restrict__ z, const VT* __restrict__ p,
                                            const VT* __restrict__ q, DotAcc<VT>& rz, DotAcc<VT>& rr) {
  VT rv[G], zv[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int64_t k = a * G + g;
    x[k] += alpha * p[k];
    rv[g] = r[k] - alpha * q[k];
    r[k] = rv[g];
  }
  apply_prec<G, VT>(prec, a, rv, zv);
#pragma unroll
  for (int g = 0; g < G; ++g) {
    z[a * G + g] = zv[g];
    rz.fma(rv[g], zv[g]);
    rr.fma(rv[g], rv[g]);
  }
}

// The same update for the 3x3-block FP32 layout, four nodes (twelve values,
// three 16-byte vectors per array; 36 inverse-block values, nine vectors) per
// thread step, all loads issued before any store.  Nodes [lo, hi), lo a
// multiple of 4.
__device__ __forceinline__ void node_update_b3(const float* __restrict__ minv, int64_t lo, int64_t hi, float alpha,
                                               float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
                                               const float* __restrict__ p, const float* __restrict__ q,
                                               DotAcc<float>& rz, DotAcc<float>& rr) {
  const int64_t g_lo = lo >> 2, g_full = hi >> 2;  // groups [g_lo, g_full) are complete
  for (int64_t gi = g_lo + threadIdx.x; gi < g_full; gi += blockDim.x) {
    float4 xv[3], pv[3], rv[3], qv[3], mv[9];
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      xv[u] = reinterpret_cast<const float4*>(x)[gi * 3 + u];
      pv[u] = reinterpret_cast<const float4*>(p)[gi * 3 + u];
      rv[u] = reinterpret_cast<const float4*>(r)[gi * 3 + u];
      qv[u] = reinterpret_cast<const float4*>(q)[gi * 3 + u];
    }
#pragma unroll
    for (int u = 0; u < 9; ++u) mv[u] = reinterpret_cast<const float4*>(minv)[gi * 9 + u];
    const float* pf = reinterpret_cast<const float*>(pv);
    const float* qf = reinterpret_cast<const float*>(qv);
    const float* mf = reinterpret_cast<const float*>(mv);
    float* xf = reinterpret_cast<float*>(xv);
    float* rf = reinterpret_cast<float*>(rv);
    float zf[12];
#pragma unroll
    for (int e = 0; e < 12; ++e) {
      xf[e] += alpha * pf[e];
      rf[e] = rf[e] - alpha * qf[e];
    }
#pragma unroll
    for (int nd = 0; nd < 4; ++nd) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        float t = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) t = fmaf(mf[nd * 9 + i * 3 + j], rf[nd * 3 + j], t);
        zf[nd * 3 + i] = t;
      }
    }
#pragma unroll
    for (int e = 0; e < 12; ++e) {
      rz.fma(rf[e], zf[e]);
      rr.fma(rf[e], rf[e]);
    }
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      reinterpret_cast<float4*>(x)[gi * 3 + u] = xv[u];
      reinterpret_cast<float4*>(r)[gi * 3 + u] = rv[u];
      reinterpret_cast<float4*>(z)[gi * 3 + u] = make_float4(zf[4 * u], zf[4 * u + 1], zf[4 * u + 2], zf[4 * u + 3]);
    }
  }
  for (int64_t a = max(lo, g_full * 4) + threadIdx.x; a < hi; a += blockDim.x)
    node_update<3, float>(minv, a, alpha, x, r, z, p, q, rz, rr);
}

// ---- TMA bulk-copy pipeline for the sliced FP32 matrix (one ring per warp)
// Ring shape: 4 slot-rows x 2 stages timed best of {2x4, 4x2, 3x3} on the
// 1M-unknown cube (the compile-time knobs keep the other shapes buildable).
#ifndef TFG_TMA_STAGES
#define TFG_TMA_STAGES 2
#endif
#ifndef TFG_TMA_ROWS
#define TFG_TMA_ROWS 4
#endif
constexpr int kTmaStages = TFG_TMA_STAGES;  // ring depth per warp
constexpr int kTmaRows = TFG_TMA_ROWS;      // slot-rows (32 rows x 1 block slot) per stage
constexpr int kSlotVal = 32 * 9 * 4;  // value bytes of a 3x3 slot-row
constexpr int kSlotCol = 32 * 4;      // column bytes of a slot-row
constexpr int kStageBytes = kTmaRows * (kSlotVal + kSlotCol);
constexpr int kWarpRing = 128 + kTmaStages * kStageBytes;  // barriers + buffers
constexpr int kTmaSmem = (kPThreads / 32) * kWarpRing;
constexpr long long kMbarSpin = 2000000000LL;  // clock cycles a stage wait may last

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kMbarSpin) return false;
  }
}

// One stage: nrows slot-rows of values then columns, both 16-byte aligned
// (slice starts are multiples of 32 slots), completing on the stage barrier.
__device__ __forceinline__ void tma_stage(uint32_t bar, uint32_t dst, const float* sval, const int32_t* col,
                                          int64_t slot0, int nrows, uint64_t policy) {
  const uint32_t bv = (uint32_t)(nrows * kSlotVal), bc = (uint32_t)(nrows * kSlotCol);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bv + bc) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst),
      "l"(sval + slot0 * 9), "r"(bv), "r"(bar), "l"(policy)
      : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst + bv),
      "l"(col + slot0), "r"(bc), "r"(bar), "l"(policy)
      : "memory");
}

// Chunk iterator over a warp's slices s = first, first + stride, ... < end.
struct ChunkIt {
  int64_t s;
  int64_t end;
  int64_t stride;
  int k0;
  __device__ bool valid() const { return s < end; }
  __device__ void advance(const int64_t* sell_base) {
    const int len = (int)((sell_base[s + 1] - sell_base[s]) >> 5);
    k0 += kTmaRows;
    if (k0 >= len) {
      k0 = 0;
      s += stride;
      // skip empty slices
      while (s < end && sell_base[s + 1] == sell_base[s]) s += stride;
    }
  }
};

template <int G, typename VT, int MODE>
__global__ void __launch_bounds__(kPThreads, MODE == 1 ? 1 : 2) k_pcg_persistent(PersistParams P) {
  using ACC = DotAcc<VT>;
  __shared__ double wsum[kPThreads / 32][2];
  __shared__ float ys[kPThreads / 32][G][32];
  __shared__ VT sh_alpha, sh_beta;
  __shared__ int sh_stop;
  Ctrl* c = P.ctrl;
  if (ctrl_idle(c)) return;
  const int cta = blockIdx.x, NC = gridDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  VT* __restrict__ x = (VT*)P.x;
  VT* __restrict__ r = (VT*)P.r;
  VT* __restrict__ z = (VT*)P.z;
  VT* __restrict__ p = (VT*)P.p;
  VT* __restrict__ q = (VT*)P.q;
  const uint64_t stream = l2_policy(false);
  // rows owned by this CTA: equal shares of the stored entries (CSR) or of
  // the stored slot-rows (sliced layout), the SpMV being the dominant phase
  int64_t row_lo, row_hi, s_lo = 0, s_hi = 0;
  if constexpr (G == 1) {
    const int64_t total = P.row_ptr[P.n_rows];
    row_lo = lower_bound_i64(P.row_ptr, P.n_rows, total * cta / NC);
    row_hi = cta == NC - 1 ? P.n_rows : lower_bound_i64(P.row_ptr, P.n_rows, total * (cta + 1) / NC);
  } else {
    const int64_t ns = (P.n_rows + 31) >> 5;
    const int64_t total = P.row_ptr[ns];
    s_lo = lower_bound_i64(P.row_ptr, ns, total * cta / NC);
    s_hi = cta == NC - 1 ? ns : lower_bound_i64(P.row_ptr, ns, total * (cta + 1) / NC);
    row_lo = min(s_lo * 32, P.n_rows);
    row_hi = min(s_hi * 32, P.n_rows);
  }
  // per-warp TMA ring (MODE 1): barriers then kTmaStages stage buffers
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  unsigned char* ring_base = dyn_smem + (size_t)warp * kWarpRing + 128;
  const uint32_t bars = smem_u32(dyn_smem + (size_t)warp * kWarpRing);
  const uint32_t bufs = smem_u32(ring_base);
  int64_t issued = 0, consumed = 0;
  bool ring_ok = true;
  // this warp's chunks (whole slices s_lo + warp, + NW, ...), cycled across
  // iterations: the producer stays kTmaStages chunks ahead of the consumer,
  // so the first chunks of the next iteration stream in during the vector
  // phases and barriers
  ChunkIt first{s_lo + warp, s_hi, NW, 0};
  ChunkIt prod = first;
  if constexpr (MODE == 1) {
    if (lane == 0) {
      for (int st = 0; st < kTmaStages; ++st) mbar_init(bars + 8u * st);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    while (first.valid() && P.row_ptr[first.s + 1] == P.row_ptr[first.s]) first.s += NW;
    prod = first;
    if (G == 3 && first.valid()) {
      for (int st = 0; st < kTmaStages; ++st) {
        if (lane == 0) {
          const int len = (int)((P.row_ptr[prod.s + 1] - P.row_ptr[prod.s]) >> 5);
          tma_stage(bars + 8u * st, bufs + (uint32_t)st * kStageBytes, (const float*)P.val, P.col,
                    P.row_ptr[prod.s] + (int64_t)prod.k0 * 32, min(kTmaRows, len - prod.k0), stream);
        }
        prod.advance(P.row_ptr);
        if (!prod.valid()) prod = first;
        ++issued;
      }
    }
  }
  // long CSR rows of this CTA, ascending (warp ballots read in warp order);
  // rows from long_cut on are left to the lane groups
  __shared__ int64_t long_rows[kLongMax];
  __shared__ unsigned long_mask[kPThreads / 32];
  __shared__ double long_sum[kPThreads / 32];
  __shared__ int n_long;
  __shared__ int64_t long_cut;
  if constexpr (G == 1) {
    if (threadIdx.x == 0) {
      n_long = 0;
      long_cut = row_hi;
    }
    __syncthreads();
    for (int64_t b = row_lo; b < row_hi; b += blockDim.x) {
      const int64_t row = b + threadIdx.x;
      const bool lg = row < row_hi && P.row_ptr[row + 1] - P.row_ptr[row] > kLongRow;
      const unsigned m = __ballot_sync(0xffffffffu, lg);
      if (lane == 0) long_mask[warp] = m;
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int w = 0; w < NW; ++w) {
          unsigned mm = long_mask[w];
          while (mm) {
            const int64_t rw = b + w * 32 + (__ffs(mm) - 1);
            mm &= mm - 1;
            if (long_cut != row_hi) break;
            if (n_long < kLongMax) long_rows[n_long++] = rw;
            else long_cut = rw;
          }
        }
      }
      __syncthreads();
    }
  }
  double rz = c->rz;        // thread 0 keeps the CG scalars
  double alpha_d = 0.0;
  long long iters = c->iters;
  const long long max_iter = c->max_iter;
  const double tol2bb = c->tol2_lo, delta2 = c->delta2, rr_ref = c->rr_ref;
  const int mixed = c->mixed;
  // two barriers per iteration on the TMA path (direction update inside the
  // SpMV).  Only there: q then carries A p by recurrence, and its drift from
  // the explicit product grows with the length of a launch.  Mixed solves
  // relaunch at every FP64 replacement (q = A p afresh) and inner Newton
  // solves stop at 1e-6; a plain FP64 solve is one long launch, where the
  // drift measurably degrades tight tolerances, so it keeps three barriers.
  constexpr bool kCarry = MODE == 1 && G == 3 && sizeof(VT) == 4;
  bool carry = false;
  if (threadIdx.x == 0) sh_beta = (VT)0;
  __syncthreads();
  while (true) {
    // ---- phase A: q = A p on own rows, partial p.q
    ACC pq[1];
    if constexpr (G == 1) {
      // groups of kCsrTpr lanes per scalar row, 32 / kCsrTpr rows per warp
      constexpr int TPR = kCsrTpr;
      const double* val = (const double*)P.val;
      const int sub = lane % TPR;
      const int64_t gid = (int64_t)warp * (32 / TPR) + lane / TPR;
      const int64_t n_groups = (int64_t)NW * (32 / TPR);
      for (int64_t row0 = row_lo; row0 < row_hi; row0 += n_groups) {
        const int64_t row = row0 + gid;
        double sacc = 0.0;
        bool own = false;
        if (row < row_hi) {
          const int64_t rs = P.row_ptr[row], re = P.row_ptr[row + 1];
          own = re - rs <= kLongRow || row >= long_cut;
          if (own) {
#pragma unroll 4
            for (int64_t j = rs + sub; j < re; j += TPR)
              sacc += ld_l2(val + j, stream) * (double)p[ld_l2(P.col + j, stream)];
          }
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) sacc += __shfl_down_sync(0xffffffffu, sacc, o, TPR);
        if (sub == 0 && own) {
          q[row] = (VT)sacc;
          pq[0].fma(p[row], (VT)sacc);
        }
      }
      // the listed long rows: all threads, warp trees, then warp sums in order
      const int nl = n_long;
      for (int i = 0; i < nl; ++i) {
        const int64_t row = long_rows[i];
        const int64_t rs = P.row_ptr[row], re = P.row_ptr[row + 1];
        double s = 0.0;
#pragma unroll 4
        for (int64_t j = rs + threadIdx.x; j < re; j += blockDim.x)
          s += ld_l2(val + j, stream) * (double)p[ld_l2(P.col + j, stream)];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) long_sum[warp] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
          double t = 0.0;
          for (int w = 0; w < NW; ++w) t += long_sum[w];
          q[row] = (VT)t;
          pq[0].fma(p[row], (VT)t);
        }
        __syncthreads();
      }
    } else if constexpr (MODE == 1 && G == 3) {
      // TMA ring per warp: whole slices per warp, no cross-warp reduction.
      // First iteration of a launch: q = A p.  Later ones fold the direction
      // update into the SpMV: gather z, then q = A z + beta q and
      // p = z + beta p on the rows just produced (q carries A p by
      // recurrence within a launch, so one barrier less per iteration).
      const float* sval = (const float*)P.val;
      const VT* gsrc = carry ? z : p;
      const VT beta = sh_beta;
      if (ring_ok && first.valid()) {
        ChunkIt cons = first;
        float y[G];
#pragma unroll
        for (int i = 0; i < G; ++i) y[i] = 0.f;
        while (cons.valid()) {
          const int slot = (int)(consumed % kTmaStages);
          const uint32_t parity = (uint32_t)((consumed / kTmaStages) & 1);
          if (!mbar_wait(bars + 8u * slot, parity)) {
            ring_ok = false;
            atomicExch(&c->bar_error, 1);
            break;
          }
          const int len = (int)((P.row_ptr[cons.s + 1] - P.row_ptr[cons.s]) >> 5);
          const int nr = min(kTmaRows, len - cons.k0);
          const float* vb = (const float*)(ring_base + (size_t)slot * kStageBytes);
          const int32_t* cb = (const int32_t*)(ring_base + (size_t)slot * kStageBytes + (size_t)nr * kSlotVal);
          // all gathers of the stage in flight before the products
          float xs[kTmaRows][G];
#pragma unroll
          for (int rr = 0; rr < kTmaRows; ++rr) {
            if (rr < nr) {
              const int64_t cc = cb[rr * 32 + lane];
#pragma unroll
              for (int j = 0; j < G; ++j) xs[rr][j] = (float)gsrc[cc * G + j];
            }
          }
#pragma unroll
          for (int rr = 0; rr < kTmaRows; ++rr) {
            if (rr < nr) {
#pragma unroll
              for (int i = 0; i < G; ++i)
#pragma unroll
                for (int j = 0; j < G; ++j) y[i] = fmaf(vb[(rr * 9 + i * G + j) * 32 + lane], xs[rr][j], y[i]);
            }
          }
          ++consumed;
          if (cons.k0 + nr >= len) {  // slice done: rows of this warp
            const int64_t a = cons.s * 32 + lane;
            if (a < P.n_rows) {
#pragma unroll
              for (int i = 0; i < G; ++i) {
                const int64_t k = a * G + i;
                VT qv = (VT)y[i], pv = p[k];
                if (carry) {
                  qv = fmaf(beta, q[k], qv);
                  pv = fmaf(beta, pv, z[k]);
                  p[k] = pv;
                }
                q[k] = qv;
                pq[0].fma(pv, qv);
              }
            }
#pragma unroll
            for (int i = 0; i < G; ++i) y[i] = 0.f;
          }
          cons.advance(P.row_ptr);
          // refill the slot just read with the chunk kTmaStages ahead
          __syncwarp();
          if (lane == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const int ps = (int)(issued % kTmaStages);
            const int plen = (int)((P.row_ptr[prod.s + 1] - P.row_ptr[prod.s]) >> 5);
            tma_stage(bars + 8u * ps, bufs + (uint32_t)ps * kStageBytes, sval, P.col,
                      P.row_ptr[prod.s] + (int64_t)prod.k0 * 32, min(kTmaRows, plen - prod.k0), stream);
          }
          prod.advance(P.row_ptr);
          if (!prod.valid()) prod = first;
          ++issued;
        }
      }
    } else {
      constexpr int DD = G * G;
      const float* sval = (const float*)P.val;
      const int NG = NW / kPKS, grp = warp / kPKS, kofs = warp % kPKS;
      for (int64_t base = s_lo; base < s_hi; base += NG) {
        const int64_t s = base + grp;
        float y[G];
#pragma unroll
        for (int i = 0; i < G; ++i) y[i] = 0.f;
        if (s < s_hi) {
          const int64_t b0 = P.row_ptr[s];
          const int len = (int)((P.row_ptr[s + 1] - b0) >> 5);
          const int32_t* cp = P.col + b0 + lane;
          const float* vp = sval + b0 * DD + lane;
#pragma unroll 2
          for (int k = kofs; k < len; k += kPKS) {
            const int64_t cc = ld_l2(cp + (int64_t)k * 32, stream);
            const float* vk = vp + (int64_t)k * DD * 32;
            float m[DD];
#pragma unroll
            for (int e = 0; e < DD; ++e) m[e] = ld_l2(vk + e * 32, stream);
            float xv[G];
#pragma unroll
            for (int j = 0; j < G; ++j) xv[j] = (float)p[cc * G + j];
#pragma unroll
            for (int i = 0; i < G; ++i)
#pragma unroll
              for (int j = 0; j < G; ++j) y[i] = fmaf(m[i * G + j], xv[j], y[i]);
          }
        }
#pragma unroll
        for (int i = 0; i < G; ++i) ys[warp][i][lane] = y[i];
        __syncthreads();
        if (kofs == 0 && s < s_hi) {
          const int64_t a = s * 32 + lane;
          if (a < P.n_rows) {
#pragma unroll
            for (int i = 0; i < G; ++i) {
              float t = ys[warp][i][lane];
#pragma unroll
              for (int v = 1; v < kPKS; ++v) t += ys[warp + v][i][lane];
              q[a * G + i] = (VT)t;
              pq[0].fma(p[a * G + i], (VT)t);
            }
          }
        }
        __syncthreads();
      }
    }
    cta_partials<1, ACC>(pq, P.partial + 3 * cta, wsum);
    const bool ok1 = grid_barrier<1>(c, P.spin_limit, P.partial, 0, [&](const double* sm) {
      const double pq_tot = sm[0];
      if (pq_tot == 0.0 || !isfinite(pq_tot)) {
        sh_stop = 1;
        if (cta == 0) {
          c->done = isfinite(pq_tot) ? kDoneBreakdown : kDoneNonFinite;
          c->iters = iters;
        }
      } else {
        sh_stop = 0;
        alpha_d = (double)(VT)(rz / pq_tot);
        sh_alpha = (VT)alpha_d;
      }
    });
    if (!ok1 || sh_stop) break;
    const VT alpha = sh_alpha;
    // ---- phase B: x += alpha p, r -= alpha q, z = M r on own rows
    ACC rzrr[2];
    if constexpr (G == 3 && sizeof(VT) == 4 && MODE == 1) {
      node_update_b3((const float*)P.prec, row_lo, row_hi, (float)alpha, (float*)x, (float*)r, (float*)z,
                     (const float*)p, (const float*)q, rzrr[0], rzrr[1]);
    } else {
      for (int64_t a = row_lo + threadIdx.x; a < row_hi; a += blockDim.x)
        node_update<G, VT>(P.prec, a, alpha, x, r, z, p, q, rzrr[0], rzrr[1]);
    }
    cta_partials<2, ACC>(rzrr, P.partial + 3 * cta + 1, wsum);
    const bool ok2 = grid_barrier<2>(c, P.spin_limit, P.partial, 1, [&](const double* sm) {
      const double rz_new = sm[0], rr = sm[1];
      iters += 1;
      int stop = 0;  // 1 done, 2 replace
      int done = kDoneNo;
      if (!isfinite(rr) || !isfinite(rz_new)) {
        stop = 1;
        done = kDoneNonFinite;
      } else if (mixed) {
        if (rr <= tol2bb || rr <= delta2 * rr_ref) stop = 2;
      } else if (rr <= tol2bb) {
        stop = 1;
        done = kDoneConverged;
      }
      if (!stop && iters >= max_iter) {
        stop = 1;
        done = kDoneMaxIter;
      }
      if (stop) {
        sh_stop = 1;
        if (cta == 0) {
          c->iters = iters;
          c->rr = rr;
          c->alpha = alpha_d;
          c->rz_new = rz_new;
          if (stop == 2) c->replace = 1;
          else c->done = done;
        }
        return;
      }
      sh_stop = 0;
      const VT beta = (VT)(rz_new / rz);
      sh_beta = beta;
      rz = rz_new;
      if (cta == 0) {
        c->rz = rz;
        c->rr = rr;
        c->iters = iters;
        c->beta = (double)beta;
      }
    });
    if (!ok2 || sh_stop) break;
    if constexpr (kCarry) {
      carry = true;  // the next SpMV applies p = z + beta p itself
    } else {
      // ---- phase C: p = z + beta p on own rows
      direction_update<VT, MODE == 1 ? 4 : 2>(p, z, sh_beta, row_lo * G, row_hi * G);
      if (!grid_barrier<0>(c, P.spin_limit, nullptr, 0, [](const double*) {})) break;
    }
  }
  if constexpr (MODE == 1) {
    // wait for this warp's prefetched chunks before the CTA exits
    while (consumed < issued) {
      mbar_wait(bars + 8u * (uint32_t)(consumed % kTmaStages), (uint32_t)((consumed / kTmaStages) & 1));
      ++consumed;
    }
  }
  if (cta == 0 && threadIdx.x == 0 && *(volatile int*)&c->bar_error) c->done = kDoneBarrierTimeout;
}

// ------------------------------------------------------------------ MINRES --
// Jacobi-preconditioned MINRES (Paige & Saunders, SIAM J. Numer. Anal. 12,
// 1975) on the FP64 CSR matrix: the reference's GPU `method="minres"`
// (sparse.py:405-412, CuPy's minres with a Jacobi M).  Three kernels per
// iteration; every scalar of the Lanczos / Givens recurrences lives in the
// control block and is updated by the last-arriving CTA, so the host only
// reads the control block between chunks of iterations.  Buffers rotate
// (r1, r2, y and w1, w2, w) by host-side indexing instead of copies.
// Stops when the preconditioned residual estimate phibar <= rtol * beta1.
struct MrCtrl {
  double beta1, beta, oldb, alfa, dbar, epsln, oldeps, phibar, phi, cs, sn, gamma, delta, tnorm2;
  double rtol;
  long long itn, max_iter;
  int done;
  int pending;  // a w / x update of the last iteration has not been applied yet
  unsigned int counter;
};

__device__ __forceinline__ bool mr_idle(const MrCtrl* c) { return (*(volatile const int*)&c->done) != 0; }

// x = 0, r1 = r2 = b, pz = M b; beta1 = sqrt(b . M b).
__global__ void __launch_bounds__(256) k_mr_init(int64_t n, const double* __restrict__ b, const double* __restrict__ dinv,
                                                 double* __restrict__ x, double* __restrict__ r1,
                                                 double* __restrict__ r2, double* __restrict__ pz,
                                                 double* __restrict__ partial, MrCtrl* c) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double bi = b[i], zi = dinv[i] * bi;
    x[i] = 0.0;
    r1[i] = bi;
    r2[i] = bi;
    pz[i] = zi;
    s += bi * zi;
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (arrive_last(&c->counter)) {
    const double t = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      c->counter = 0;
      if (!(t >= 0.0) || !isfinite(t)) {
        c->done = kDoneNonFinite;
      } else {
        const double b1 = sqrt(t);
        c->beta1 = c->beta = c->phibar = b1;
        c->oldb = c->dbar = c->epsln = c->oldeps = c->phi = c->gamma = c->delta = c->tnorm2 = c->alfa = 0.0;
        c->cs = -1.0;
        c->sn = 0.0;
        c->itn = 0;
        c->pending = 0;
        c->done = b1 == 0.0 ? kDoneConverged : kDoneNo;
      }
    }
  }
}

// Pending update of the previous iteration (w = (v - oldeps w1 - delta w2) /
// gamma, x += phi w) with that iteration's v, then v = pz / beta for this one.
__global__ void __launch_bounds__(256) k_mr_step(int64_t n, double* __restrict__ v, const double* __restrict__ pz,
                                                 const double* __restrict__ w1, const double* __restrict__ w2,
                                                 double* __restrict__ w, double* __restrict__ x, MrCtrl* c) {
  const int pending = c->pending;
  const bool run = !mr_idle(c);
  if (!pending && !run) return;
  const double oldeps = c->oldeps, delta = c->delta, gamma = c->gamma, phi = c->phi, s = 1.0 / c->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (pending) {
      const double wi = (v[i] - oldeps * w1[i] - delta * w2[i]) / gamma;
      w[i] = wi;
      x[i] += phi * wi;
    }
    if (run) v[i] = s * pz[i];
  }
  if (arrive_last(&c->counter) && threadIdx.x == 0) {
    c->counter = 0;
    c->pending = 0;
  }
}

// y = A v - (beta / oldb) r1 (scalar CSR, TPR lanes per row); alfa = v . y.
template <int TPR>
__global__ void __launch_bounds__(256) k_mr_spmv(int64_t n, const int64_t* __restrict__ row_ptr,
                                                 const int32_t* __restrict__ col, const double* __restrict__ val,
                                                 const double* __restrict__ v, const double* __restrict__ r1,
                                                 double* __restrict__ y, double* __restrict__ partial, MrCtrl* c) {
  __shared__ double red[32];
  if (mr_idle(c)) return;
  const double f = c->itn >= 1 ? c->beta / c->oldb : 0.0;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = t / TPR;
  const int sub = (int)(t % TPR);
  double s = 0.0, vy = 0.0;
  if (row < n) {
    const int64_t rs = row_ptr[row], re = row_ptr[row + 1];
    for (int64_t j = rs + sub; j < re; j += TPR) s += val[j] * v[col[j]];
  }
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
  if (row < n && sub == 0) {
    const double yi = s - f * r1[row];
    y[row] = yi;
    vy = v[row] * yi;
  }
  vy = block_sum(vy, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = vy;
  if (arrive_last(&c->counter)) {
    const double a = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      c->counter = 0;
      c->alfa = a;
      if (!isfinite(a)) c->done = kDoneNonFinite;
    }
  }
}

// y -= (alfa / beta) r2; pz = M y; beta' = sqrt(y . pz); then the Lanczos
// and Givens recurrences and the stopping test (last CTA).
__global__ void __launch_bounds__(256) k_mr_update(int64_t n, double* __restrict__ y, const double* __restrict__ r2,
                                                   const double* __restrict__ dinv, double* __restrict__ pz,
                                                   double* __restrict__ partial, MrCtrl* c) {
  __shared__ double red[32];
  if (mr_idle(c)) return;
  const double f = c->alfa / c->beta;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double yi = y[i] - f * r2[i];
    const double zi = dinv[i] * yi;
    y[i] = yi;
    pz[i] = zi;
    s += yi * zi;
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (arrive_last(&c->counter)) {
    const double t = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      c->counter = 0;
      if (!(t >= 0.0) || !isfinite(t)) {  // M must be positive definite
        c->done = isfinite(t) ? kDoneBreakdown : kDoneNonFinite;
      } else {
        const double alfa = c->alfa;
        c->oldb = c->beta;
        const double beta = sqrt(t);
        c->beta = beta;
        c->tnorm2 += alfa * alfa + c->oldb * c->oldb + beta * beta;
        // previous rotation on the new column
        c->oldeps = c->epsln;
        const double delta = c->cs * c->dbar + c->sn * alfa;
        const double gbar = c->sn * c->dbar - c->cs * alfa;
        c->epsln = c->sn * beta;
        c->dbar = -c->cs * beta;
        // new rotation
        double gamma = sqrt(gbar * gbar + beta * beta);
        if (gamma < 1e-300) gamma = 1e-300;
        c->cs = gbar / gamma;
        c->sn = beta / gamma;
        c->phi = c->cs * c->phibar;
        c->phibar = c->sn * c->phibar;
        c->delta = delta;
        c->gamma = gamma;
        c->pending = 1;
        c->itn += 1;
        if (c->phibar <= c->rtol * c->beta1 || beta == 0.0) c->done = kDoneConverged;
        else if (c->itn >= c->max_iter) c->done = kDoneMaxIter;
      }
    }
  }
}

// Diagnostic for the bounded waits: CTA 1 leaves at once, CTA 0 waits at a
// grid barrier of two CTAs that therefore never completes; the wait must run
// out after spin_limit cycles, set bar_error and return.
__global__ void k_diag_barrier(Ctrl* c, long long spin_limit) {
  if (blockIdx.x != 0) return;
  grid_barrier<0>(c, spin_limit, nullptr, 0, [](const double*) {});
}

// ------------------------------------------------------------- host driver --
constexpr int kThreads = 256;

// SM count of the current device (cached per host thread).
static int sm_count() {
  static thread_local int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 132;
  }
  return n;
}

// Bytes of matrix data kept resident in L2 across CG iterations (read with
// evict_last); the rest streams with evict_first.  TORCHFEM_GB300_L2_KEEP_MB
// overrides the default for experiments.
static int64_t l2_keep_bytes() {
  static int64_t keep = -1;
  if (keep < 0) {
    const char* e = getenv("TORCHFEM_GB300_L2_KEEP_MB");
    keep = (int64_t)((e ? atof(e) : 0.0) * 1e6);
    if (keep < 0) keep = 0;
  }
  return keep;
}

static unsigned vec_grid(int64_t n) {
  const int64_t cap = (int64_t)sm_count() * 4;
  const int64_t need = (n + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min(cap, need));
}

static unsigned sell_grid(int64_t n_rows) {
  const int64_t ns = (n_rows + 31) / 32;
  const int64_t cap = (int64_t)sm_count() * 16;
  return (unsigned)std::max<int64_t>(1, std::min(cap, ns));
}

static int read_ctrl(Ctrl* d, Ctrl* h, cudaStream_t st) {
  if (cudaMemcpyAsync(h, d, sizeof(Ctrl), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return check_cuda("read_ctrl");
  if (cudaStreamSynchronize(st) != cudaSuccess) return check_cuda("read_ctrl sync");
  return FEM_OK;
}

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

static int64_t spmv_grid(const fem_matrix* A) {
  if (A->format == FEM_FMT_CSR_F64) return grid_for(A->n_rows * kCsrTpr, kThreads);
  return sell_grid(A->n_rows);
}

// Persistent CG: CTAs per SM from the occupancy calculator (cached).
template <int G, typename VT, int MODE>
static int persistent_blocks() {
  static thread_local int blocks = 0;
  if (blocks == 0) {
    const int smem = MODE == 1 ? kTmaSmem : 0;
    if (MODE == 1)
      cudaFuncSetAttribute(k_pcg_persistent<G, VT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pcg_persistent<G, VT, MODE>, kPThreads, smem) !=
            cudaSuccess ||
        occ < 1)
      occ = 1;
    blocks = occ * sm_count();
  }
  return blocks;
}

// The TMA-pipelined SpMV serves the FP32 3x3 sliced layout (the mixed path).
static int g_tma_spmv = -1;
static bool use_tma_spmv() {
  if (g_tma_spmv < 0) {
    const char* e = getenv("TORCHFEM_GB300_TMA");
    g_tma_spmv = (e && strcmp(e, "0") == 0) ? 0 : 1;
  }
  return g_tma_spmv == 1;
}

// Upper bound on the persistent grid (at most 2048 / kPThreads CTAs per SM).
static int64_t persistent_grid_bound() { return (int64_t)sm_count() * (2048 / kPThreads); }

static int g_cg_path = -1;  // 1 persistent, 0 per-iteration kernels
static thread_local bool g_persistent_refused = false;
constexpr int FEM_COOP_TOO_LARGE = 100;  // internal: cooperative grid refused

static bool use_persistent() {
  if (g_cg_path < 0) {
    const char* e = getenv("TORCHFEM_GB300_CG");
    g_cg_path = (e && strcmp(e, "kernels") == 0) ? 0 : 1;
  }
  return g_cg_path == 1;
}

static int64_t max_grid(const fem_matrix* A) {
  return std::max<int64_t>(std::max<int64_t>(spmv_grid(A), grid_for(A->n, kThreads)),
                           persistent_grid_bound());
}

static int status_of(int done) {
  switch (done) {
    case kDoneConverged: return FEM_OK;
    case kDoneMaxIter: return FEM_NOT_CONVERGED;
    case kDoneNonFinite: return FEM_NONFINITE;
    case kDoneBreakdown: return FEM_BREAKDOWN;
    case kDoneBarrierTimeout: return FEM_CUDA_ERROR;
    default: return FEM_NOT_CONVERGED;
  }
}

static int validate_matrix(const fem_matrix* A) {
  if (!A || A->n <= 0) {
    set_last_error("fem_pcg: empty matrix");
    return FEM_INVALID;
  }
  if (A->format == FEM_FMT_CSR_F64) {
    if (A->block != 1 || A->n_rows != A->n) {
      set_last_error("fem_pcg: CSR needs block 1 and n_rows == n");
      return FEM_INVALID;
    }
  } else if (A->format == FEM_FMT_SELL_F32) {
    if (A->block < 2 || A->block > 3 || A->n_rows * A->block != A->n) {
      set_last_error("fem_pcg: sliced blocks need block 2 or 3 and n_rows * block == n");
      return FEM_INVALID;
    }
  } else {
    set_last_error("fem_pcg: unknown matrix format %d", A->format);
    return FEM_INVALID;
  }
  return FEM_OK;
}

// Optional CUDA-event timing of the SpMV launches (fem_set_timing).
constexpr int kMaxChunk = 64;
int g_timing = 0;  // CUDA-event timing of the CG (fem_set_timing), read by the multigrid CG too

struct SpmvTimer {
  cudaEvent_t ev[2 * kMaxChunk];
  bool ready = false;
  double ms = 0.0;
  long long timed = 0;
  int init() {
    if (ready) return FEM_OK;
    for (int i = 0; i < 2 * kMaxChunk; ++i)
      if (cudaEventCreate(&ev[i]) != cudaSuccess) return check_cuda("event create");
    ready = true;
    return FEM_OK;
  }
  // Sums the durations of the first `active` SpMV launches of a chunk.
  void collect(int active) {
    for (int c = 0; c < active && c < kMaxChunk; ++c) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, ev[2 * c], ev[2 * c + 1]) == cudaSuccess) {
        ms += t;
        timed += 1;
      }
    }
  }
  // no destructor: the events live until the process exits, when the CUDA
  // runtime may already be gone
};

static thread_local SpmvTimer g_timer;

// One CG iteration (SpMV, update, direction) on the working precision;
// slot >= 0 brackets the SpMV with the timer's events.
template <int G, typename VT>
static void launch_iteration(const fem_matrix* A, VT* x, VT* r, VT* z, VT* p, VT* q, double* partial,
                             Ctrl* ctrl, cudaStream_t st, int slot = -1) {
  if (slot >= 0) cudaEventRecord(g_timer.ev[2 * slot], st);
  if constexpr (G == 1) {
    k_spmv_csr<kCsrTpr><<<grid_for(A->n_rows * kCsrTpr, kThreads), kThreads, 0, st>>>(
        A->n_rows, A->row_ptr, A->col, (const double*)A->val, (const double*)p, (double*)q,
        partial, ctrl, l2_keep_bytes() / 12);
  } else {
    k_spmv_sell<G><<<sell_grid(A->n_rows), kSellWarps * 32, 0, st>>>(
        A->n_rows, A->row_ptr, A->col, (const float*)A->val, (const float*)p, (float*)q, partial,
        ctrl, l2_keep_bytes() / (4 * G * G + 4));
  }
  ::tfg::note_launch();
  if (slot >= 0) cudaEventRecord(g_timer.ev[2 * slot + 1], st);
  const int64_t ng = A->n / G;
  k_update<G, VT><<<vec_grid(ng), kThreads, 0, st>>>(ng, x, r, p, q, z, A->precond, partial, ctrl);
  ::tfg::note_launch();
  k_pupdate<VT><<<vec_grid(A->n), kThreads, 0, st>>>(A->n, z, p, ctrl);
  ::tfg::note_launch();
}

// One cooperative launch of the persistent CG kernel on the given vectors.
template <int G, typename VT>
static int launch_persistent(const fem_matrix* A, VT* x, VT* r, VT* z, VT* p, VT* q, double* partial,
                             Ctrl* ctrl, cudaStream_t st) {
  PersistParams P;
  P.n = A->n;
  P.n_rows = A->n_rows;
  P.row_ptr = A->row_ptr;
  P.col = A->col;
  P.val = A->val;
  P.prec = A->precond;
  P.x = x;
  P.r = r;
  P.z = z;
  P.p = p;
  P.q = q;
  P.partial = partial;
  P.ctrl = ctrl;
  P.spin_limit = 2000000000LL;  // about one second of clock cycles
  void* args[] = {&P};
  cudaError_t e;
  if (G == 3 && use_tma_spmv()) {
    const int blocks = persistent_blocks<G, VT, 1>();
    e = cudaLaunchCooperativeKernel((const void*)k_pcg_persistent<G, VT, 1>, dim3(blocks), dim3(kPThreads), args,
                                    kTmaSmem, st);
  } else {
    const int blocks = persistent_blocks<G, VT, 0>();
    e = cudaLaunchCooperativeKernel((const void*)k_pcg_persistent<G, VT, 0>, dim3(blocks), dim3(kPThreads), args,
                                    0, st);
  }
  ::tfg::note_launch();
  if (e != cudaSuccess) {
    set_last_error("persistent CG launch: %s", cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorCooperativeLaunchTooLarge ? FEM_COOP_TOO_LARGE : FEM_CUDA_ERROR;
  }
  return FEM_OK;
}

// Runs CG iterations until the control block reports done or a pending
// replacement: persistent kernel by default, per-iteration kernels when
// TORCHFEM_GB300_CG=kernels.  Updates *h from the device.
template <int G, typename VT>
static int iterate(const fem_matrix* A, VT* x, VT* r, VT* z, VT* p, VT* q, double* partial, Ctrl* ctrl,
                   Ctrl* h, bool timing, int* chunk, cudaStream_t st) {
  const long long before = h->iters;
  if (use_persistent() && !g_persistent_refused) {
    if (timing) cudaEventRecord(g_timer.ev[0], st);
    int rc = launch_persistent<G, VT>(A, x, r, z, p, q, partial, ctrl, st);
    if (rc == FEM_COOP_TOO_LARGE) {
      // the device cannot hold the whole grid at once (shared with other
      // work): run this solve with per-iteration kernels instead
      g_persistent_refused = true;
      return iterate<G, VT>(A, x, r, z, p, q, partial, ctrl, h, timing, chunk, st);
    }
    if (rc) return rc;
    if (timing) cudaEventRecord(g_timer.ev[1], st);
    rc = read_ctrl(ctrl, h, st);
    if (rc) return rc;
    if (timing) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, g_timer.ev[0], g_timer.ev[1]) == cudaSuccess) {
        g_timer.ms += t;
        g_timer.timed += h->iters - before;
      }
    }
    if (h->done == kDoneNo && !h->replace) {
      set_last_error("persistent CG returned without progress");
      return FEM_CUDA_ERROR;
    }
    return FEM_OK;
  }
  for (int c = 0; c < *chunk; ++c)
    launch_iteration<G, VT>(A, x, r, z, p, q, partial, ctrl, st, timing ? c : -1);
  TFG_CHECK_LAUNCH("CG iterate");
  int rc = read_ctrl(ctrl, h, st);
  if (rc) return rc;
  if (timing) g_timer.collect((int)(h->iters - before));
  *chunk = std::min(*chunk * 2, kMaxChunk);
  return FEM_OK;
}

struct Vecs {
  Ctrl* ctrl;
  void *x, *r, *z, *p, *q;
  double* partial;
  double* y64;
  double* fe;
  void* gather_ws;
};

static size_t layout(const fem_matrix* A, int64_t fe_len, Vecs* v, void* ws) {
  const size_t vt = (A->format == FEM_FMT_CSR_F64) ? sizeof(double) : sizeof(float);
  const int64_t n = A->n;
  char* base = reinterpret_cast<char*>(ws);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* ptr = base ? base + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  Vecs t;
  t.ctrl = reinterpret_cast<Ctrl*>(take(sizeof(Ctrl)));
  t.x = take(n * vt);
  t.r = take(n * vt);
  t.z = take(n * vt);
  t.p = take(n * vt);
  t.q = take(n * vt);
  t.partial = reinterpret_cast<double*>(take(sizeof(double) * 3 * (max_grid(A) + 1)));
  t.y64 = fe_len > 0 ? reinterpret_cast<double*>(take(sizeof(double) * n)) : nullptr;
  t.fe = fe_len > 0 ? reinterpret_cast<double*>(take(sizeof(double) * fe_len)) : nullptr;
  t.gather_ws = nullptr;
  if (v) *v = t;
  return off;
}

template <int G, typename VT>
static int run_pcg(const fem_matrix* A, const double* b, double* x, double rtol, int64_t max_iter,
                   const Vecs& v, fem_solve_info* info, cudaStream_t st, bool timing_on) {
  Ctrl h;
  memset(&h, 0, sizeof(h));
  h.max_iter = max_iter;
  h.mixed = 0;
  h.rscale = 1.0;
  if (cudaMemcpyAsync(v.ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return check_cuda("fem_pcg ctrl");
  VT* xv = (G == 1) ? reinterpret_cast<VT*>(x) : reinterpret_cast<VT*>(v.x);
  const int64_t ng = A->n / G;
  g_persistent_refused = false;
  if (sizeof(VT) == 4) {  // FP32 vectors iterate on b scaled to near unit norm
    k_bnorm<<<vec_grid(A->n), kThreads, 0, st>>>(A->n, b, v.partial, v.ctrl);
    ::tfg::note_launch();
  }
  k_init<G, VT><<<grid_for(ng, kThreads), kThreads, 0, st>>>(
      ng, b, xv, (VT*)v.r, (VT*)v.z, (VT*)v.p, A->precond, v.partial, v.ctrl, rtol * rtol);
      ::tfg::note_launch();
  TFG_CHECK_LAUNCH("fem_pcg init");
  int rc = read_ctrl(v.ctrl, &h, st);
  if (rc) return rc;
  const bool timing = timing_on && g_timer.init() == FEM_OK;
  if (timing) {
    g_timer.ms = 0.0;
    g_timer.timed = 0;
  }
  int chunk = 8;
  while (h.done == kDoneNo) {
    rc = iterate<G, VT>(A, xv, (VT*)v.r, (VT*)v.z, (VT*)v.p, (VT*)v.q, v.partial, v.ctrl, &h, timing,
                        &chunk, st);
    if (rc) return rc;
  }
  if (G != 1) k_copy_cast<<<grid_for(A->n, kThreads), kThreads, 0, st>>>(A->n, (const float*)v.x, x, v.ctrl);
  ::tfg::note_launch();
  TFG_CHECK_LAUNCH("fem_pcg finish");
  if (info) {
    info->iterations = h.iters;
    info->replacements = 0;
    info->rel_residual = h.bb > 0 ? sqrt(h.rr / h.bb) / h.rscale : 0.0;
    info->status = status_of(h.done);
    info->spmv_ms = timing ? g_timer.ms : 0.0;
    info->spmv_timed = timing ? g_timer.timed : 0;
  }
  if (h.done == kDoneBarrierTimeout)
    set_last_error("persistent CG: a grid-barrier or TMA-stage wait ran out (barrier timeout) after %lld iterations",
                   h.iters);
  else if (h.done != kDoneConverged)
    set_last_error("CG did not converge: %lld iterations, relative residual %.3e, code %d", h.iters,
                   h.bb > 0 ? sqrt(h.rr / h.bb) / h.rscale : 0.0, h.done);
  return status_of(h.done);
}

// y = A x in FP64 over the FP64 copy of the sliced matrix A32 describes
// (A32->n_rows block rows of A32->block DOFs).
int sell_apply64(const fem_matrix* A32, const double* sval64, const double* x, double* y, cudaStream_t st) {
  const int64_t nr = A32->n_rows;
  const int64_t ns = (nr + 31) / 32;
  if (ns == 0) return FEM_OK;
  switch (A32->block) {
    case 1:
      k_sell_apply64<1><<<(unsigned)((ns + kApplyW - 1) / kApplyW), kApplyW * 32, 0, st>>>(
          nr, ns, A32->row_ptr, A32->col, sval64, x, y);
      break;
    case 2:
      k_sell_apply64<2><<<(unsigned)ns, kApplyW * 32, 0, st>>>(nr, ns, A32->row_ptr, A32->col, sval64, x, y);
      break;
    case 3:
      k_sell_apply64<3><<<(unsigned)ns, kApplyW * 32, 0, st>>>(nr, ns, A32->row_ptr, A32->col, sval64, x, y);
      break;
    default:
      set_last_error("FP64 sliced apply: block size %d", A32->block);
      return FEM_INVALID;
  }
  ::tfg::note_launch();
  return check_cuda("FP64 sliced apply");
}

}  // namespace tfg

using namespace tfg;

extern "C" {

void fem_set_timing(int enable) { g_timing = enable; }

void fem_set_cg_path(int path) {
  g_cg_path = path == 0 ? 0 : 1;
  if (path == 1) g_tma_spmv = 1;
  if (path == 2) g_tma_spmv = 0;
}
int fem_get_cg_path(void) { return use_persistent() ? (use_tma_spmv() ? 1 : 2) : 0; }

int fem_assemble_csr(const fem_blocks* B, int ke_dtype, const void* ke, const int64_t* row_ptr,
                     const uint8_t* con_mask, double* val, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (B->dim < 1 || B->dim > 6) {
    set_last_error("fem_assemble_csr: DOFs per node must be 1..6");
    return FEM_INVALID;
  }
  if (B->n_blocks == 0) return FEM_OK;
  const unsigned g = grid_for(B->n_blocks, 128);
  if (B->dim > 3) {  // shells: six DOFs per node
    if (ke_dtype == FEM_F64)
      k_assemble<double, double, false, 6><<<g, 128, 0, st>>>(
          B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row,
          B->inc_ptr, (const double*)ke, row_ptr, con_mask, val, nullptr, nullptr);
    else
      k_assemble<float, double, false, 6><<<g, 128, 0, st>>>(
          B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row,
          B->inc_ptr, (const float*)ke, row_ptr, con_mask, val, nullptr, nullptr);
    ::tfg::note_launch();
    return check_cuda("fem_assemble_csr");
  }
  if (ke_dtype == FEM_F64)
    k_assemble<double, double, false><<<g, 128, 0, st>>>(
        B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row,
        B->inc_ptr, (const double*)ke, row_ptr, con_mask, val, nullptr, nullptr);
  else
    k_assemble<float, double, false><<<g, 128, 0, st>>>(
        B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row,
        B->inc_ptr, (const float*)ke, row_ptr, con_mask, val, nullptr, nullptr);
        ::tfg::note_launch();
  return check_cuda("fem_assemble_csr");
}

size_t fem_sell_workspace_bytes(int64_t n_nod) {
  const int64_t ns = (n_nod + 31) / 32;
  return (size_t)(ns + 1) * sizeof(int64_t) + scan_workspace_bytes(ns);
}

int fem_sell_layout(const fem_blocks* B, int64_t* sell_base, int64_t* n_slots, void* ws,
                    size_t ws_bytes, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (ws_bytes < fem_sell_workspace_bytes(B->n_nod)) {
    set_last_error("fem_sell_layout: workspace too small");
    return FEM_INVALID;
  }
  const int64_t ns = (B->n_nod + 31) / 32;
  int64_t* len = reinterpret_cast<int64_t*>(ws);
  k_sell_len<<<grid_for(ns, kThreads), kThreads, 0, st>>>(B->nbr_ptr, B->n_nod, len);
  ::tfg::note_launch();
  int rc = scan_exclusive(len, sell_base, ns, len + ns + 1, st);
  if (rc) return rc;
  if (cudaMemcpyAsync(n_slots, sell_base + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("fem_sell_layout sync");
  return check_cuda("fem_sell_layout");
}

int fem_sell_columns(const fem_blocks* B, const int64_t* sell_base, int32_t* col, void* stream) {
  cudaStream_t st = as_stream(stream);
  const int64_t ns = (B->n_nod + 31) / 32;
  k_sell_cols<<<grid_for(ns * 32, kThreads), kThreads, 0, st>>>(B->nbr_ptr, B->nbr, B->n_nod, sell_base, col);
  ::tfg::note_launch();
  return check_cuda("fem_sell_columns");
}

int fem_assemble_sell(const fem_blocks* B, int ke_dtype, const void* ke, const uint8_t* con_mask,
                      const int64_t* sell_base, int64_t n_slots, float* sval, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (B->dim < 1 || B->dim > 3) {
    set_last_error("fem_assemble_sell: dim must be 1..3");
    return FEM_INVALID;
  }
  cudaMemsetAsync(sval, 0, sizeof(float) * n_slots * B->dim * B->dim, st);
  if (B->n_blocks == 0) return check_cuda("fem_assemble_sell");
  const unsigned g = grid_for(B->n_blocks, 128);
  if (ke_dtype == FEM_F64)
    k_assemble<double, double, true><<<g, 128, 0, st>>>(
        B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row,
        B->inc_ptr, (const double*)ke, nullptr, con_mask, nullptr, sell_base, sval);
  else
    k_assemble<float, float, true><<<g, 128, 0, st>>>(
        B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row,
        B->inc_ptr, (const float*)ke, nullptr, con_mask, nullptr, sell_base, sval);
  ::tfg::note_launch();
  return check_cuda("fem_assemble_sell");
}

int fem_assemble_sell_pair(const fem_blocks* B, const double* ke, const uint8_t* con_mask,
                           const int64_t* sell_base, int64_t n_slots, float* sval, double* sval64,
                           void* stream) {
  cudaStream_t st = as_stream(stream);
  if (B->dim < 1 || B->dim > 3) {
    set_last_error("fem_assemble_sell_pair: dim must be 1..3");
    return FEM_INVALID;
  }
  if (!sval || !sval64) {
    set_last_error("fem_assemble_sell_pair: sval and sval64 are required");
    return FEM_INVALID;
  }
  const size_t nv = (size_t)n_slots * B->dim * B->dim;
  cudaMemsetAsync(sval, 0, sizeof(float) * nv, st);
  cudaMemsetAsync(sval64, 0, sizeof(double) * nv, st);
  if (B->n_blocks == 0) return check_cuda("fem_assemble_sell_pair");
  k_assemble<double, double, true><<<grid_for(B->n_blocks, 128), 128, 0, st>>>(
      B->n_e, B->dim, B->n_blocks, B->nbr_ptr, B->nbr, B->blk_ptr, B->contrib, B->blk_row, B->inc_ptr, ke,
      nullptr, con_mask, nullptr, sell_base, sval, sval64);
  ::tfg::note_launch();
  return check_cuda("fem_assemble_sell_pair");
}

int fem_sell_apply64(const fem_matrix* A32, const double* sval64, const double* x, double* y, void* stream) {
  if (!A32 || A32->format != FEM_FMT_SELL_F32 || !sval64) {
    set_last_error("fem_sell_apply64: needs the FP32 sliced matrix's layout and its FP64 copy");
    return FEM_INVALID;
  }
  return sell_apply64(A32, sval64, x, y, as_stream(stream));
}

int fem_jacobi(const double* val, const int64_t* diag_map, int64_t n, double* inv_diag,
               int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  k_jacobi<<<grid_for(n, kThreads), kThreads, 0, st>>>(val, diag_map, n, inv_diag, status);
  ::tfg::note_launch();
  return check_cuda("fem_jacobi");
}

int fem_block_jacobi(const fem_blocks* B, const float* sval, const int64_t* sell_base,
                     float* inv_blocks, int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  k_block_jacobi<<<grid_for(B->n_nod, kThreads), kThreads, 0, st>>>(
      sval, sell_base, B->nbr_ptr, B->diag_blk, B->n_nod, B->dim, inv_blocks, status);
                                                                    ::tfg::note_launch();
  return check_cuda("fem_block_jacobi");
}

size_t fem_pcg_workspace_bytes(const fem_matrix* A) {
  if (validate_matrix(A) != FEM_OK) return 0;
  return layout(A, 0, nullptr, nullptr);
}

int fem_pcg(const fem_matrix* A, const double* b, double* x, double rtol, int64_t max_iter, void* ws,
            size_t ws_bytes, fem_solve_info* info, void* stream) {
  int rc = validate_matrix(A);
  if (rc) return rc;
  if (ws_bytes < fem_pcg_workspace_bytes(A)) {
    set_last_error("fem_pcg: workspace too small");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  Vecs v;
  layout(A, 0, &v, ws);
  const bool timing = g_timing != 0;
  if (A->format == FEM_FMT_CSR_F64) return run_pcg<1, double>(A, b, x, rtol, max_iter, v, info, st, timing);
  if (A->block == 2) return run_pcg<2, float>(A, b, x, rtol, max_iter, v, info, st, timing);
  return run_pcg<3, float>(A, b, x, rtol, max_iter, v, info, st, timing);
}

static int64_t op_fe_len(const fem_operator64* op) {
  int ne, d, nip;
  if (etype_info(op->mesh->etype, &ne, &d, &nip) != FEM_OK) return -1;
  if (op->mesh->dof_per_node > 0) d = op->mesh->dof_per_node;
  return op->mesh->n_elem * ne * d;
}

size_t fem_apply64_workspace_bytes(const fem_operator64* op) {
  const int64_t fl = op_fe_len(op);
  if (fl < 0) return 0;
  return align256(sizeof(double) * (fl > 0 ? fl : 1));
}

int fem_apply64(const fem_operator64* op, const double* x, double* y, void* ws, size_t ws_bytes,
                void* stream) {
  if (ws_bytes < fem_apply64_workspace_bytes(op)) {
    set_last_error("fem_apply64: workspace too small");
    return FEM_INVALID;
  }
  double* fe = reinterpret_cast<double*>(ws);
  int rc = fem_element_force(op->mesh, op->mat, x, op->con_mask, nullptr, 2, nullptr, nullptr, fe,
                             nullptr, nullptr, nullptr, stream);
  if (rc) return rc;
  return fem_gather_nodal(op->mesh, fe, nullptr, op->con_mask, 2, x, y, nullptr, nullptr, 0, stream);
}

size_t fem_pcg_mixed_workspace_bytes(const fem_matrix* A32, const fem_operator64* op) {
  if (validate_matrix(A32) != FEM_OK || A32->format != FEM_FMT_SELL_F32) return 0;
  const int64_t fl = op_fe_len(op);
  if (fl < 0) return 0;
  return layout(A32, fl > 0 ? fl : 1, nullptr, nullptr);
}

int fem_pcg_mixed(const fem_matrix* A, const fem_operator64* op, const double* b, double* x,
                  double rtol, double delta, int64_t max_iter, void* ws, size_t ws_bytes,
                  fem_solve_info* info, void* stream) {
  int rc = validate_matrix(A);
  if (rc) return rc;
  if (A->format != FEM_FMT_SELL_F32) {
    set_last_error("fem_pcg_mixed: needs an FP32 sliced-block matrix");
    return FEM_INVALID;
  }
  const size_t need = fem_pcg_mixed_workspace_bytes(A, op);
  if (need == 0 || ws_bytes < need) {
    set_last_error("fem_pcg_mixed: workspace too small");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  Vecs v;
  layout(A, op_fe_len(op), &v, ws);
  Ctrl h;
  memset(&h, 0, sizeof(h));
  h.max_iter = max_iter;
  h.mixed = 1;
  h.delta2 = delta * delta;
  h.rscale = 1.0;
  if (cudaMemcpyAsync(v.ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return check_cuda("fem_pcg_mixed ctrl");
  const int G = A->block;
  const int64_t ng = A->n / G;
  g_persistent_refused = false;
  float *xl = (float*)v.x, *r = (float*)v.r, *z = (float*)v.z, *p = (float*)v.p, *q = (float*)v.q;
  cudaMemsetAsync(x, 0, sizeof(double) * A->n, st);
  k_bnorm<<<vec_grid(A->n), kThreads, 0, st>>>(A->n, b, v.partial, v.ctrl);
  ::tfg::note_launch();
  if (G == 2)
    k_init<2, float><<<grid_for(ng, kThreads), kThreads, 0, st>>>(ng, b, xl, r, z, p, A->precond,
                                                                  v.partial, v.ctrl, rtol * rtol);
  else
    k_init<3, float><<<grid_for(ng, kThreads), kThreads, 0, st>>>(ng, b, xl, r, z, p, A->precond,
                                                                  v.partial, v.ctrl, rtol * rtol);
                                                                  ::tfg::note_launch();
  TFG_CHECK_LAUNCH("fem_pcg_mixed init");
  rc = read_ctrl(v.ctrl, &h, st);
  if (rc) return rc;
  const bool timing = g_timing && g_timer.init() == FEM_OK;
  g_timer.ms = 0.0;
  g_timer.timed = 0;
  int chunk = 8;
  // stagnation guard: the FP64 residual must halve within kStallReplacements
  // replacements, else FP32 storage cannot refine this system
  constexpr int kStallReplacements = 8;
  double best_rr = -1.0;
  int stalled = 0;
  while (h.done == kDoneNo) {
    if (h.replace) {
      // FP64 reliable update: x += x_lo; r = b - A x (matrix-free FP64).
      k_fold<<<grid_for(A->n, kThreads), kThreads, 0, st>>>(A->n, x, xl, v.ctrl);
      ::tfg::note_launch();
      if (op->sell_val64) {
        rc = sell_apply64(A, op->sell_val64, x, v.y64, st);
      } else {
        rc = fem_element_force(op->mesh, op->mat, x, op->con_mask, nullptr, 2, nullptr, nullptr, v.fe,
                               nullptr, nullptr, nullptr, stream);
        if (!rc)
          rc = fem_gather_nodal(op->mesh, v.fe, nullptr, op->con_mask, 2, x, v.y64, nullptr, nullptr, 0,
                                stream);
      }
      if (rc) return rc;
      if (G == 2)
        k_replace<2><<<grid_for(ng, kThreads), kThreads, 0, st>>>(ng, b, v.y64, r, z, A->precond,
                                                                  v.partial, v.ctrl);
      else
        k_replace<3><<<grid_for(ng, kThreads), kThreads, 0, st>>>(ng, b, v.y64, r, z, A->precond,
                                                                  v.partial, v.ctrl);
                                                                  ::tfg::note_launch();
      k_pupdate<float><<<vec_grid(A->n), kThreads, 0, st>>>(A->n, z, p, v.ctrl);
      ::tfg::note_launch();
      TFG_CHECK_LAUNCH("fem_pcg_mixed replace");
      rc = read_ctrl(v.ctrl, &h, st);
      if (rc) return rc;
      if (h.done == kDoneNo) {
        if (best_rr < 0.0 || h.rr_true < 0.25 * best_rr) {
          best_rr = h.rr_true;
          stalled = 0;
        } else if (++stalled >= kStallReplacements) {
          set_last_error("mixed CG stagnated at relative residual %.3e after %lld iterations: FP32 "
                         "storage cannot refine this system; use precision fp64",
                         h.bb > 0 ? sqrt(h.rr_true / h.bb) : 0.0, h.iters);
          k_fold<<<grid_for(A->n, kThreads), kThreads, 0, st>>>(A->n, x, xl, v.ctrl);
          ::tfg::note_launch();
          if (info) {
            info->iterations = h.iters;
            info->replacements = h.replacements;
            info->rel_residual = h.bb > 0 ? sqrt(h.rr_true / h.bb) : 0.0;
            info->status = FEM_NOT_CONVERGED;
          }
          return FEM_NOT_CONVERGED;
        }
      }
      continue;
    }
    if (G == 2) rc = iterate<2, float>(A, xl, r, z, p, q, v.partial, v.ctrl, &h, timing, &chunk, st);
    else rc = iterate<3, float>(A, xl, r, z, p, q, v.partial, v.ctrl, &h, timing, &chunk, st);
    if (rc) return rc;
  }
  // fold whatever correction is left (max-iter exit) into x
  k_fold<<<grid_for(A->n, kThreads), kThreads, 0, st>>>(A->n, x, xl, v.ctrl);
  ::tfg::note_launch();
  TFG_CHECK_LAUNCH("fem_pcg_mixed finish");
  rc = read_ctrl(v.ctrl, &h, st);
  if (rc) return rc;
  if (info) {
    info->iterations = h.iters;
    info->replacements = h.replacements;
    info->rel_residual = h.bb > 0 ? sqrt(h.rr_true / h.bb) : 0.0;
    info->status = status_of(h.done);
    info->spmv_ms = timing ? g_timer.ms : 0.0;
    info->spmv_timed = timing ? g_timer.timed : 0;
  }
  if (h.done == kDoneBarrierTimeout)
    set_last_error("persistent CG: a grid-barrier or TMA-stage wait ran out (barrier timeout) after %lld iterations",
                   h.iters);
  else if (h.done != kDoneConverged)
    set_last_error("mixed CG did not converge: %lld iterations, relative residual %.3e, code %d",
                   h.iters, h.bb > 0 ? sqrt(h.rr_true / h.bb) : 0.0, h.done);
  return status_of(h.done);
}

}  // extern "C"

// ---------------------------------------------------------- diagnostics --
extern "C" {

int fem_diag_barrier_timeout(void* ws, size_t ws_bytes, long long spin_limit, void* stream) {
  if (!ws || ws_bytes < sizeof(Ctrl) || spin_limit <= 0) {
    set_last_error("fem_diag_barrier_timeout: needs a workspace of %zu bytes and a positive limit", sizeof(Ctrl));
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  Ctrl* c = reinterpret_cast<Ctrl*>(ws);
  if (cudaMemsetAsync(c, 0, sizeof(Ctrl), st) != cudaSuccess) return check_cuda("fem_diag_barrier_timeout memset");
  k_diag_barrier<<<2, 32, 0, st>>>(c, spin_limit);
  note_launch();
  TFG_CHECK_LAUNCH("fem_diag_barrier_timeout");
  int err = 0;
  if (cudaMemcpyAsync(&err, &c->bar_error, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("fem_diag_barrier_timeout read");
  if (err) {
    set_last_error("persistent CG: a grid-barrier or TMA-stage wait ran out (barrier timeout)");
    return FEM_CUDA_ERROR;
  }
  return FEM_OK;
}

size_t fem_diag_workspace_bytes(void) { return sizeof(Ctrl); }

}  // extern "C"

// --------------------------------------------------------------- MINRES --
namespace tfg {

struct MrVecs {
  MrCtrl* ctrl;
  double *v, *pz, *R[3], *W[3];
  double* partial;
};

static size_t mr_layout(int64_t n, unsigned grid, MrVecs* v, void* ws) {
  char* base = reinterpret_cast<char*>(ws);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* ptr = base ? base + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  MrVecs t;
  t.ctrl = reinterpret_cast<MrCtrl*>(take(sizeof(MrCtrl)));
  t.v = reinterpret_cast<double*>(take(n * sizeof(double)));
  t.pz = reinterpret_cast<double*>(take(n * sizeof(double)));
  for (int i = 0; i < 3; ++i) t.R[i] = reinterpret_cast<double*>(take(n * sizeof(double)));
  for (int i = 0; i < 3; ++i) t.W[i] = reinterpret_cast<double*>(take(n * sizeof(double)));
  t.partial = reinterpret_cast<double*>(take(sizeof(double) * (grid + 1)));
  if (v) *v = t;
  return off;
}

static unsigned mr_grid(const fem_matrix* A) {
  return std::max<unsigned>(vec_grid(A->n), grid_for(A->n_rows * kCsrTpr, kThreads));
}

}  // namespace tfg

extern "C" {

size_t fem_minres_workspace_bytes(const fem_matrix* A) {
  if (validate_matrix(A) != FEM_OK || A->format != FEM_FMT_CSR_F64 || A->block != 1) return 0;
  return mr_layout(A->n, mr_grid(A), nullptr, nullptr);
}

int fem_minres(const fem_matrix* A, const double* b, double* x, double rtol, int64_t max_iter, void* ws,
               size_t ws_bytes, fem_solve_info* info, void* stream) {
  int rc = validate_matrix(A);
  if (rc) return rc;
  if (A->format != FEM_FMT_CSR_F64 || A->block != 1) {
    set_last_error("fem_minres: needs the FP64 scalar CSR matrix with its inverse diagonal");
    return FEM_INVALID;
  }
  const size_t need = fem_minres_workspace_bytes(A);
  if (need == 0 || ws_bytes < need) {
    set_last_error("fem_minres: workspace too small");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  const int64_t n = A->n;
  MrVecs v;
  mr_layout(n, mr_grid(A), &v, ws);
  MrCtrl h;
  memset(&h, 0, sizeof(h));
  h.rtol = rtol;
  h.max_iter = max_iter;
  if (cudaMemcpyAsync(v.ctrl, &h, sizeof(MrCtrl), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return check_cuda("fem_minres ctrl");
  for (int i = 0; i < 3; ++i) cudaMemsetAsync(v.W[i], 0, sizeof(double) * n, st);
  const double* dinv = (const double*)A->precond;
  const unsigned vg = vec_grid(n);
  k_mr_init<<<vg, kThreads, 0, st>>>(n, b, dinv, x, v.R[0], v.R[1], v.pz, v.partial, v.ctrl);
  note_launch();
  TFG_CHECK_LAUNCH("fem_minres init");
  if (cudaMemcpyAsync(&h, v.ctrl, sizeof(MrCtrl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("fem_minres read");
  const unsigned sg = grid_for(A->n_rows * kCsrTpr, kThreads);
  int64_t k = 0;
  int chunk = 8;
  while (h.done == kDoneNo) {
    for (int c = 0; c < chunk; ++c, ++k) {
      k_mr_step<<<vg, kThreads, 0, st>>>(n, v.v, v.pz, v.W[k % 3], v.W[(k + 1) % 3], v.W[(k + 2) % 3], x, v.ctrl);
      k_mr_spmv<kCsrTpr><<<sg, kThreads, 0, st>>>(A->n_rows, A->row_ptr, A->col, (const double*)A->val, v.v,
                                                  v.R[k % 3], v.R[(k + 2) % 3], v.partial, v.ctrl);
      k_mr_update<<<vg, kThreads, 0, st>>>(n, v.R[(k + 2) % 3], v.R[(k + 1) % 3], dinv, v.pz, v.partial, v.ctrl);
      note_launch();
      note_launch();
      note_launch();
    }
    TFG_CHECK_LAUNCH("fem_minres iterate");
    if (cudaMemcpyAsync(&h, v.ctrl, sizeof(MrCtrl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return check_cuda("fem_minres read");
    chunk = std::min(chunk * 2, 256);
  }
  // the last iteration's w / x update
  k_mr_step<<<vg, kThreads, 0, st>>>(n, v.v, v.pz, v.W[k % 3], v.W[(k + 1) % 3], v.W[(k + 2) % 3], x, v.ctrl);
  note_launch();
  TFG_CHECK_LAUNCH("fem_minres finish");
  if (cudaStreamSynchronize(st) != cudaSuccess) return check_cuda("fem_minres sync");
  if (info) {
    info->iterations = h.itn;
    info->replacements = 0;
    info->rel_residual = h.beta1 > 0 ? h.phibar / h.beta1 : 0.0;
    info->status = status_of(h.done);
    info->spmv_ms = 0.0;
    info->spmv_timed = 0;
  }
  if (h.done != kDoneConverged)
    set_last_error("MINRES did not converge: %lld iterations, preconditioned residual %.3e, code %d", h.itn,
                   h.beta1 > 0 ? h.phibar / h.beta1 : 0.0, h.done);
  return status_of(h.done);
}

}  // extern "C"

// ------------------------------------------------- allocation-free CG solve --
// fem_pcg_static: the same preconditioned CG as fem_pcg, for callers that
// cannot allocate device memory at the point where they solve — an embedding
// host behind an FFI that has no binding to a CUDA allocator, or a control
// loop where cudaMalloc's implicit synchronisation, or its failure under
// memory pressure, is not acceptable.  Its scratch (CG vectors, reduction
// partials, control block) lives in one file-scope device array that every
// GPU loading this library holds until the process exits.  All calls share
// that array: calls that overlap on the GPU (different streams or host
// threads on the same device) race on it and must be serialised by the
// caller.  Everything the solve reads from the array is rewritten at the
// start of each call, so the contents left by a previous call do not matter.
namespace tfg {

constexpr size_t kStaticScratchBytes = size_t(6) << 20;  // 6 MiB per device
constexpr int64_t kStaticMaxUnknowns = 131072;

static __device__ __align__(256) unsigned char g_pcg_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
static void* g_scratch_ptr[kMaxDevices] = {nullptr};
static std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device.  The array's
// name is a host-side stand-in, so the address is looked up once per device
// with that device current and kept for the life of the process: the entry
// point must not be used on a device after cudaDeviceReset (or any other
// re-creation of its primary context) in this process.
static int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_cuda("fem_pcg_static: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("fem_pcg_static: device id %d beyond %d", dev, kMaxDevices);
    return FEM_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_last_error("fem_pcg_static: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return FEM_CUDA_ERROR;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return FEM_OK;
}

}  // namespace tfg

extern "C" {

int64_t fem_pcg_static_max_unknowns(void) { return tfg::kStaticMaxUnknowns; }

int fem_pcg_static(const fem_matrix* A, const double* b, double* x, double rtol, int64_t max_iter,
                   fem_solve_info* info, void* stream) {
  int rc = validate_matrix(A);
  if (rc) return rc;
  if (A->n > kStaticMaxUnknowns) {
    set_last_error("fem_pcg_static: %lld unknowns exceed the static workspace limit of %lld unknowns; "
                   "use fem_pcg with a caller workspace",
                   (long long)A->n, (long long)kStaticMaxUnknowns);
    return FEM_BOUNDS;
  }
  const size_t need = fem_pcg_workspace_bytes(A);
  if (need > kStaticScratchBytes) {
    set_last_error("fem_pcg_static: the solve needs %zu bytes of scratch, more than the static workspace "
                   "limit of %zu bytes; use fem_pcg with a caller workspace",
                   need, kStaticScratchBytes);
    return FEM_BOUNDS;
  }
  void* ws = nullptr;
  rc = static_scratch(&ws);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  Vecs v;
  layout(A, 0, &v, ws);
  // no SpMV event timing here: the timer creates CUDA events on first use
  // (and the process-wide timing switch is left alone)
  if (A->format == FEM_FMT_CSR_F64) rc = run_pcg<1, double>(A, b, x, rtol, max_iter, v, info, st, false);
  else if (A->block == 2) rc = run_pcg<2, float>(A, b, x, rtol, max_iter, v, info, st, false);
  else rc = run_pcg<3, float>(A, b, x, rtol, max_iter, v, info, st, false);
  return rc;
}

}  // extern "C"
