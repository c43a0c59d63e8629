// Smoothed-aggregation algebraic multigrid (SA-AMG) for the FP32 block systems
// of the mixed-precision solver, and the multigrid-preconditioned CG built on
// it.  This is the GPU counterpart of the preconditioner the reference builds
// for its iterative solves: on the CPU pyamg.smoothed_aggregation_solver(A, B,
// smooth="jacobi") with B the rigid-body modes of FEM.compute_B
// (src/torchfem/sparse.py:495-507, src/torchfem/base.py:316-344), on the GPU
// AmgX aggregation AMG (src/torchfem/amgx.py:62-91).
//
// Published methods, restated for this library:
//  - aggregation: roots form a distance-2 maximal independent set chosen with
//    fixed pseudo-random priorities, then two passes attach every remaining
//    node to the aggregate of a neighbour (Bell, Dalton & Olson, "Exposing
//    fine-grained parallelism in algebraic multigrid methods", SIAM J. Sci.
//    Comput. 34 (2012) C123-C152);
//  - tentative prolongator T: per aggregate, an orthonormal basis of the
//    near-null space (rigid-body modes with constrained components removed)
//    from a Cholesky-QR with rank drop; its triangular factor is the coarse
//    near-null space of the next level (Vanek, Mandel & Brezina, Computing 56
//    (1996) 179-196);
//  - prolongator smoothing P = (I - w D^-1 A) T, w = 4 / (3 rho(D^-1 A)), D
//    the block diagonal (pyamg's smooth="jacobi" default);
//  - Galerkin coarse operators A_c = P^T A P;
//  - smoothing: Chebyshev polynomial of degree 2 in D^-1 A on
//    [0.1, 1.1] rho (Adams, Brezina, Hu & Tuminaro, J. Comput. Phys. 188 (2003)
//    593-610), rho estimated by 12 CG-Lanczos steps; a symmetric smoother, so
//    the V-cycle is a symmetric positive definite preconditioner and plain CG
//    applies (the reference's CPU path also runs CG);
//  - coarsest level (at most 96 unknowns): dense inverse.
//
// Determinism: no floating-point atomics; every sum runs in a fixed order and
// the aggregation priorities are fixed, so hierarchy and iterates are identical
// run to run.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "fem_common.cuh"

namespace tfg {

int etype_info(int etype, int* ne, int* d, int* nip);
extern int g_timing;  // fem_set_timing
int g_amg_half = 1;   // FP16 smoothing copy of the level-0 matrix (fem_amg_set_half_smoother)
int g_amg_fused = 1;  // coarse levels as one cooperative launch per V-cycle (fem_amg_set_fused_cycle)
int g_amg_tma = 1;    // level-0 slices streamed by bulk copies (fem_amg_set_level0_tma)
int g_amg_pdl = 1;    // programmatic dependent launch in the CG iteration (fem_amg_set_pdl)
int sell_apply64(const fem_matrix* A32, const double* sval64, const double* x, double* y, cudaStream_t st);
size_t scan_workspace_bytes(int64_t n);
int scan_exclusive(const int64_t* in, int64_t* out, int64_t n, int64_t* ws, cudaStream_t st);

namespace {

constexpr int kMaxLevels = 10;
constexpr int kMaxPRow = 64;       // aggregates adjacent to one node
constexpr int kMaxAPRow = 128;     // block columns of one row of A P
constexpr int kMaxCRow = 128;      // block columns of one coarse row
constexpr int kCoarseMaxDof = 96;  // the coarsest level is inverted densely
constexpr int kLanczos = 12;       // CG-Lanczos steps of the spectral estimate
constexpr double kChebLo = 0.1, kChebHi = 1.1;
constexpr double kOmega = 4.0 / 3.0;
constexpr double kDropTol = 1e-10;  // relative pivot below which a mode is dropped
constexpr int kT = 256;             // threads of the row-parallel kernels
constexpr int kSellW = 4;           // warps sharing one 32-row slice (level 0)

int g_sm = 0;
int sm_count() {
  if (g_sm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&g_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || g_sm <= 0) g_sm = 132;
  }
  return g_sm;
}
unsigned capped(int64_t blocks_needed, int per_sm) {
  const int64_t cap = (int64_t)sm_count() * per_sm;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks_needed, cap));
}

// ------------------------------------------------------------ priorities --
// lowbias32 integer hash (C. Wellons, 2018): fixed pseudo-random priorities.
__host__ __device__ __forceinline__ uint32_t amg_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// MIS key: (state, priority, index), compared as one 64-bit word.  State 0
// (decided out, or inactive) maps to 0; 1 undecided; 2 root.
__device__ __forceinline__ uint64_t mis_key(int64_t i, int st) {
  return st == 0 ? 0ull
                 : ((uint64_t)st << 62) | ((uint64_t)(amg_hash((uint32_t)i) >> 2) << 32) | (uint64_t)(uint32_t)i;
}

__device__ __forceinline__ uint64_t join_key(int64_t j) {
  return (1ull << 63) | ((uint64_t)(amg_hash((uint32_t)j) >> 2) << 32) | (uint64_t)(uint32_t)j;
}

// ------------------------------------------------------------ control ----
enum { kRun = 0, kConverged = 1, kMaxIter = 2, kNonFinite = 3, kBreakdown = 4, kBarrierTimeout = 5 };

struct AmgCtrl {
  double rz;       // r.z of the current direction
  double pscale;   // factor on beta: 0 for a fresh start (first direction, after a replacement), else 1
  double alpha;
  double beta;
  double rr;       // ||r||^2 of the FP32 residual (scaled units)
  double rr_ref;   // rr at the last FP64 replacement
  double rr_true;  // ||b - A x||^2 of the last FP64 replacement
  double bb;
  double tol2bb;
  double rscale;   // power of two applied to the FP32 residual
  double tol2_lo;  // tol2bb * rscale^2
  double delta2;
  long long iters;
  long long max_iter;
  long long replacements;
  int done;
  int replace;
  int mixed;
  unsigned int counter;
  int lz_step;
};

__device__ __forceinline__ bool amg_idle(const AmgCtrl* c) {
  return (*(volatile const int*)&c->done) != 0 || (*(volatile const int*)&c->replace) != 0;
}

// Programmatic dependent launch on the CG iteration's chain of kernels: each
// waits for its predecessor's completion (and memory) before reading
// anything, then lets its own successor be scheduled early, so a launch's
// set-up overlaps the predecessor's tail.  Both are no-ops for a kernel
// launched without the attribute.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <int B>
__device__ __forceinline__ void block_mv(const float* __restrict__ m, const float (&v)[B], float (&out)[B]) {
#pragma unroll
  for (int a = 0; a < B; ++a) {
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < B; ++c) s = fmaf(m[a * B + c], v[c], s);
    out[a] = s;
  }
}

// N FP16 values to FP32 (4-byte loads when N is even: callers keep the start
// 4-byte aligned).
template <int N>
__device__ __forceinline__ void load_half(const __half* __restrict__ src, float (&dst)[N]) {
  if constexpr (N % 2 == 0) {
    const __half2* s2 = reinterpret_cast<const __half2*>(src);
#pragma unroll
    for (int c = 0; c < N / 2; ++c) {
      const float2 f = __half22float2(s2[c]);
      dst[2 * c] = f.x;
      dst[2 * c + 1] = f.y;
    }
  } else {
#pragma unroll
    for (int c = 0; c < N; ++c) dst[c] = __half2float(src[c]);
  }
}

// ================================================================ symbolic ==
struct Graph {
  int64_t n;
  const int64_t* ptr;
  const int32_t* idx;
};

__global__ void k_centroid(int64_t n, int dim, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double red[32];
  for (int c = 0; c < dim; ++c) {
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += x[i * dim + c];
    s = block_sum(s, red);
    if (threadIdx.x == 0) out[c] = n > 0 ? s / (double)n : 0.0;
    __syncthreads();
  }
}

__global__ void k_agg_active(int64_t n, int b, const uint8_t* __restrict__ con, uint8_t* __restrict__ active,
                             uint8_t* __restrict__ state) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool act = true;
  if (con) {
    act = false;
    for (int r = 0; r < b; ++r) act = act || !con[i * b + r];
  }
  active[i] = act;
  state[i] = act ? 1 : 0;
}

// k1[i] = largest key over the active closed neighbourhood of an active node.
__global__ void k_mis_max1(Graph g, const uint8_t* __restrict__ active, const uint8_t* __restrict__ state,
                           uint64_t* __restrict__ k1) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  uint64_t m = 0;
  if (active[i])
    for (int64_t e = g.ptr[i]; e < g.ptr[i + 1]; ++e) {
      const int32_t j = g.idx[e];
      if (active[j]) m = max(m, mis_key(j, state[j]));
    }
  k1[i] = m;
}

// Distance-2 maximum; an undecided node that holds it becomes a root, one
// that sees a root within distance 2 drops out.
__global__ void k_mis_max2(Graph g, const uint8_t* __restrict__ active, uint8_t* __restrict__ state,
                           const uint64_t* __restrict__ k1, unsigned long long* __restrict__ undecided) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool und = false;
  if (i < g.n && active[i] && state[i] == 1) {
    uint64_t m = 0;
    for (int64_t e = g.ptr[i]; e < g.ptr[i + 1]; ++e) {
      const int32_t j = g.idx[e];
      if (active[j]) m = max(m, k1[j]);
    }
    if (m == mis_key(i, 1)) state[i] = 2;
    else if ((m >> 62) == 2) state[i] = 0;
    else und = true;
  }
  const unsigned bal = __ballot_sync(0xffffffffu, und);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(undecided, (unsigned long long)__popc(bal));
}

__global__ void k_root_flags(int64_t n, const uint8_t* __restrict__ state, int64_t* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = state[i] == 2 ? 1 : 0;
}

__global__ void k_root_ids(int64_t n, const uint8_t* __restrict__ state, const int64_t* __restrict__ ids,
                           int32_t* __restrict__ agg) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) agg[i] = state[i] == 2 ? (int32_t)ids[i] : -1;
}

// An unassigned active node joins the aggregate of its assigned neighbour of
// largest (priority, index).
__global__ void k_agg_join(Graph g, const uint8_t* __restrict__ active, const int32_t* __restrict__ agg_in,
                           int32_t* __restrict__ agg_out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  int32_t a = agg_in[i];
  if (a < 0 && active[i]) {
    uint64_t best = 0;
    for (int64_t e = g.ptr[i]; e < g.ptr[i + 1]; ++e) {
      const int32_t j = g.idx[e];
      const int32_t aj = agg_in[j];
      if (aj >= 0) {
        const uint64_t k = join_key(j);
        if (k > best) {
          best = k;
          a = aj;
        }
      }
    }
  }
  agg_out[i] = a;
}

__global__ void k_count_unassigned(int64_t n, const uint8_t* __restrict__ active, const int32_t* __restrict__ agg,
                                   unsigned long long* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool bad = i < n && active[i] && agg[i] < 0;
  const unsigned bal = __ballot_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(cnt, (unsigned long long)__popc(bal));
}

// Counting sort by key, in two kernels: counts, then an unordered fill that
// k_sort_rows puts in ascending order.
__global__ void k_count_keys(int64_t n, const int32_t* __restrict__ key, int64_t* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && key[i] >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(cnt + key[i]), 1ull);
}

__global__ void k_fill_keys(int64_t n, const int32_t* __restrict__ key, int64_t* __restrict__ cursor,
                            int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && key[i] >= 0) {
    const int64_t pos = (int64_t)atomicAdd(reinterpret_cast<unsigned long long*>(cursor + key[i]), 1ull);
    out[pos] = (int32_t)i;
  }
}

// Transpose of a row pattern: counts per column, then (column -> row) fill.
__global__ void k_count_cols(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ col,
                             int64_t* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) atomicAdd(reinterpret_cast<unsigned long long*>(cnt + col[e]), 1ull);
}

__global__ void k_fill_cols(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ col,
                            int64_t* __restrict__ cursor, int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
    const int64_t pos = (int64_t)atomicAdd(reinterpret_cast<unsigned long long*>(cursor + col[e]), 1ull);
    out[pos] = (int32_t)i;
  }
}

// Warp per row: out = the row of `in` in ascending order (distinct values).
__global__ void k_sort_rows(int64_t n_rows, const int64_t* __restrict__ ptr, const int32_t* __restrict__ in,
                            int32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= n_rows) return;
  const int64_t e0 = ptr[r], e1 = ptr[r + 1];
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    const int32_t v = in[e];
    int64_t rank = 0;
    for (int64_t f = e0; f < e1; ++f) rank += in[f] < v;
    out[e0 + rank] = v;
  }
}

// Position in P of every transposed entry: the slot of coarse column I in the
// P row of fine node pt_row[e].
__global__ void k_pt_pos(int64_t n_c, const int64_t* __restrict__ pt_ptr, const int32_t* __restrict__ pt_row,
                         const int64_t* __restrict__ p_ptr, const int32_t* __restrict__ p_col,
                         int64_t* __restrict__ pt_pos) {
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n_c) return;
  for (int64_t e = pt_ptr[I]; e < pt_ptr[I + 1]; ++e) {
    const int32_t i = pt_row[e];
    int64_t pos = -1;
    for (int64_t f = p_ptr[i]; f < p_ptr[i + 1]; ++f)
      if (p_col[f] == (int32_t)I) pos = f;
    pt_pos[e] = pos;
  }
}

// Sorted insertion of v into s[0..m) (distinct values); false when full.
template <int CAP>
__device__ __forceinline__ bool insert_unique(int32_t (&s)[CAP], int& m, int32_t v) {
  int k = m;
  while (k > 0 && s[k - 1] > v) --k;
  if (k > 0 && s[k - 1] == v) return true;
  if (m == CAP) return false;
  for (int t = m; t > k; --t) s[t] = s[t - 1];
  s[k] = v;
  ++m;
  return true;
}

// P pattern: row i holds the aggregates of its active neighbours.  Count
// pass (cnt) or fill pass (col at ptr).
template <bool kFill>
__global__ void k_p_rows(Graph g, const uint8_t* __restrict__ active, const int32_t* __restrict__ agg,
                         int64_t* __restrict__ cnt, const int64_t* __restrict__ ptr, int32_t* __restrict__ col,
                         int32_t* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  int32_t s[kMaxPRow];
  int m = 0;
  if (!active || active[i])
    for (int64_t e = g.ptr[i]; e < g.ptr[i + 1]; ++e) {
      const int32_t a = agg[g.idx[e]];
      if (a >= 0 && !insert_unique(s, m, a)) {
        flag_status(status, kStatBounds);
        break;
      }
    }
  if (!kFill) {
    cnt[i] = m;
  } else {
    for (int k = 0; k < m; ++k) col[ptr[i] + k] = s[k];
  }
}

// Union pattern: row i holds the union over u in outer(i) of inner(u);
// rows of inactive nodes (active[i] == 0) stay empty.
template <int CAP, bool kFill>
__global__ void k_union_rows(int64_t n, const uint8_t* __restrict__ active, const int64_t* __restrict__ optr,
                             const int32_t* __restrict__ oidx, const int64_t* __restrict__ iptr,
                             const int32_t* __restrict__ icol, int64_t* __restrict__ cnt,
                             const int64_t* __restrict__ ptr, int32_t* __restrict__ col, int32_t* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t s[CAP];
  int m = 0;
  bool ok = !active || active[i];
  for (int64_t e = optr[i]; e < optr[i + 1] && ok; ++e) {
    const int32_t u = oidx[e];
    for (int64_t f = iptr[u]; f < iptr[u + 1]; ++f)
      if (!insert_unique(s, m, icol[f])) {
        flag_status(status, kStatBounds);
        ok = false;
        break;
      }
  }
  if (!kFill) {
    cnt[i] = m;
  } else {
    for (int k = 0; k < m; ++k) col[ptr[i] + k] = s[k];
  }
}

// Row r (component) of the near-null space of node i: rigid-body modes about
// the origin c (level 0: coordinates, constrained components zero) or the
// stored rows bn [n][B][K] (coarser levels).
template <int B, int K>
__device__ __forceinline__ void null_row(int64_t i, int r, const double* __restrict__ x, const uint8_t* __restrict__ con,
                                         const double* __restrict__ bn, const double (&c)[3], double (&row)[K]) {
  if (bn) {
#pragma unroll
    for (int k = 0; k < K; ++k) row[k] = bn[(i * B + r) * K + k];
    return;
  }
#pragma unroll
  for (int k = 0; k < K; ++k) row[k] = 0.0;
  if (con && con[i * B + r]) return;
  row[r] = 1.0;
  if constexpr (B == 3 && K == 6) {
    // columns of FEM.compute_B (base.py:322-332): (0,-z,y), (z,0,-x), (-y,x,0)
    const double px = x[i * 3] - c[0], py = x[i * 3 + 1] - c[1], pz = x[i * 3 + 2] - c[2];
    if (r == 0) {
      row[4] = pz;
      row[5] = -py;
    } else if (r == 1) {
      row[3] = -pz;
      row[5] = px;
    } else {
      row[3] = py;
      row[4] = -px;
    }
  } else if constexpr (B == 2 && K == 3) {
    // compute_B in 2D (base.py:333-338): (y, -x)
    const double px = x[i * 2] - c[0], py = x[i * 2 + 1] - c[1];
    row[2] = r == 0 ? py : -px;
  }
}

// Warp per aggregate: Gram matrix of the members' near-null rows, Cholesky
// with rank drop (the R of a modified Gram-Schmidt QR that skips dependent
// columns), T = rows of Q, and the coarse near-null rows R (expressed about
// the global origin when the fine rows were taken about the centroid).
template <int B, int K>
__global__ void __launch_bounds__(128) k_tentative(int64_t n_agg, const int64_t* __restrict__ agg_ptr,
                                                   const int32_t* __restrict__ agg_nodes,
                                                   const double* __restrict__ x, const uint8_t* __restrict__ con,
                                                   const double* __restrict__ origin, const double* __restrict__ bn,
                                                   float* __restrict__ tval, double* __restrict__ bc,
                                                   unsigned long long* __restrict__ dropped) {
  constexpr int NG = K * (K + 1) / 2;
  __shared__ double Rs[4][K][K];
  __shared__ int keep[4][K];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t a = (int64_t)blockIdx.x * 4 + w;
  if (a >= n_agg) return;
  const int64_t m0 = agg_ptr[a], m1 = agg_ptr[a + 1];
  constexpr int DC = B < 3 ? B : 3;  // coordinate components (finest level)
  double c[3] = {0.0, 0.0, 0.0};
  if (!bn) {
    // rows about the aggregate centroid: the same column space, better conditioned
#pragma unroll
    for (int d = 0; d < DC; ++d) {
      double s = 0.0;
      for (int64_t e = m0 + lane; e < m1; e += 32) s += x[(int64_t)agg_nodes[e] * B + d];
      s = warp_sum(s);
      c[d] = s / (double)(m1 - m0);
    }
  }
  double G[NG];
#pragma unroll
  for (int t = 0; t < NG; ++t) G[t] = 0.0;
  for (int64_t e = m0 + lane; e < m1; e += 32) {
    const int64_t i = agg_nodes[e];
    for (int r = 0; r < B; ++r) {
      double row[K];
      null_row<B, K>(i, r, x, con, bn, c, row);
      int t = 0;
#pragma unroll
      for (int p = 0; p < K; ++p)
#pragma unroll
        for (int q = p; q < K; ++q) G[t++] += row[p] * row[q];
    }
  }
#pragma unroll
  for (int t = 0; t < NG; ++t) G[t] = warp_sum(G[t]);
  if (lane == 0) {
    double R[K][K];
    int nd = 0;
    for (int p = 0; p < K; ++p)
      for (int q = 0; q < K; ++q) R[p][q] = 0.0;
    auto gidx = [](int p, int q) { return p * K - p * (p - 1) / 2 + (q - p); };
    for (int j = 0; j < K; ++j) {
      double d = G[gidx(j, j)];
      for (int l = 0; l < j; ++l) d -= R[l][j] * R[l][j];
      const bool kp = G[gidx(j, j)] > 0.0 && d > kDropTol * G[gidx(j, j)];
      keep[w][j] = kp;
      if (!kp) {
        ++nd;
        continue;
      }
      R[j][j] = sqrt(d);
      for (int q = j + 1; q < K; ++q) {
        double v = G[gidx(j, q)];
        for (int l = 0; l < j; ++l) v -= R[l][j] * R[l][q];
        R[j][q] = v / R[j][j];
      }
    }
    for (int p = 0; p < K; ++p)
      for (int q = 0; q < K; ++q) Rs[w][p][q] = R[p][q];
    if (nd) atomicAdd(dropped, (unsigned long long)nd);
  }
  __syncwarp();
  for (int64_t e = m0 + lane; e < m1; e += 32) {
    const int64_t i = agg_nodes[e];
    for (int r = 0; r < B; ++r) {
      double row[K], q[K];
      null_row<B, K>(i, r, x, con, bn, c, row);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        double v = row[k];
        for (int l = 0; l < k; ++l) v -= q[l] * Rs[w][l][k];
        q[k] = keep[w][k] ? v / Rs[w][k][k] : 0.0;
      }
#pragma unroll
      for (int k = 0; k < K; ++k) tval[(i * B + r) * K + k] = (float)q[k];
    }
  }
  // coarse rows: R S, with S the unit upper-triangular change from modes
  // about c to modes about the global origin (translations added to rotations)
  double S[K][K];
#pragma unroll
  for (int p = 0; p < K; ++p)
#pragma unroll
    for (int q = 0; q < K; ++q) S[p][q] = p == q ? 1.0 : 0.0;
  if (!bn) {
    const double cx = c[0] - origin[0], cy = c[1] - origin[1];
    if constexpr (B == 3 && K == 6) {
      const double cz = c[2] - origin[2];
      S[1][3] = -cz;
      S[2][3] = cy;
      S[0][4] = cz;
      S[2][4] = -cx;
      S[0][5] = -cy;
      S[1][5] = cx;
    } else if constexpr (B == 2 && K == 3) {
      S[0][2] = cy;
      S[1][2] = -cx;
    }
  }
  for (int t = lane; t < K * K; t += 32) {
    const int p = t / K, q = t % K;
    double v = 0.0;
    for (int l = 0; l < K; ++l) v += Rs[w][p][l] * S[l][q];
    bc[a * K * K + t] = v;
  }
}

// ================================================================ numeric ==
// Block (i, slot kk) of the level operator: level 0 reads the sliced FP32
// matrix, coarser levels a block CSR.
template <int B, bool kSell>
struct OpView {
  const int64_t* base;  // sell_base (kSell) or row pointers
  const float* val;
  __device__ __forceinline__ float at(int64_t i, int64_t kk, int c) const {
    if constexpr (kSell) return val[base[i >> 5] * (B * B) + (kk * (B * B) + c) * 32 + (i & 31)];
    else return val[(base[i] + kk) * (B * B) + c];
  }
};

// Slot of v in the sorted list s[0..m) by binary search (v is present).
__device__ __forceinline__ int bsearch_slot(const int32_t* s, int m, int32_t v) {
  int lo = 0, hi = m - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (s[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return (m > 0 && s[lo] == v) ? lo : -1;
}

// P = T - w D^-1 A T by contribution lists: block (i, J) of A T is the sum
// over the neighbours j of i (ascending) with aggregate J of A_ij T_j.  The
// lists (neighbour slots) are built once with the pattern; a group of 8 lanes
// sums one block's list in registers, reduces in a fixed order, then applies
// D_i^-1 and subtracts from T (T_iJ is nonzero only for J = agg(i)).
template <bool kFill>
__global__ void k_p_lists(Graph g, const int32_t* __restrict__ agg, const int64_t* __restrict__ p_ptr,
                          const int32_t* __restrict__ p_col, int64_t* __restrict__ cnt, int64_t* __restrict__ cursor,
                          int32_t* __restrict__ cl_k, int32_t* __restrict__ row) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int64_t p0 = p_ptr[i];
  const int m = (int)(p_ptr[i + 1] - p0);
  if (kFill)
    for (int s = 0; s < m; ++s) row[p0 + s] = (int32_t)i;
  if (m == 0) return;
  const int64_t nb = g.ptr[i];
  const int deg = (int)(g.ptr[i + 1] - nb);
  for (int kk = 0; kk < deg; ++kk) {
    const int32_t a = agg[g.idx[nb + kk]];
    if (a < 0) continue;
    const int s = bsearch_slot(p_col + p0, m, a);
    if (s < 0) continue;  // cannot happen: the row lists every neighbour's aggregate
    if (!kFill) cnt[p0 + s] += 1;
    else cl_k[cursor[p0 + s]++] = kk;
  }
}

template <int B, int K, bool kSell>
__global__ void __launch_bounds__(256) k_p_numeric(int64_t n_slots, Graph g, OpView<B, kSell> A,
                                                   const float* __restrict__ dinv, const int32_t* __restrict__ agg,
                                                   const float* __restrict__ tval, const int64_t* __restrict__ cl_ptr,
                                                   const int32_t* __restrict__ cl_k, const int32_t* __restrict__ row,
                                                   const int32_t* __restrict__ p_col, float* __restrict__ p_val,
                                                   float omega) {
  constexpr int BK = B * K;
  const int g8 = threadIdx.x & 7;
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const bool live = s < n_slots;
  float acc[BK];
#pragma unroll
  for (int c = 0; c < BK; ++c) acc[c] = 0.f;
  int64_t i = 0;
  if (live) {
    i = row[s];
    const int64_t nb = g.ptr[i];
    for (int64_t e = cl_ptr[s] + g8; e < cl_ptr[s + 1]; e += 8) {
      const int kk = cl_k[e];
      const int64_t j = g.idx[nb + kk];
      const float* tv = tval + j * BK;
      float a[B * B], tr[BK];
#pragma unroll
      for (int c = 0; c < B * B; ++c) a[c] = A.at(i, kk, c);
#pragma unroll
      for (int c = 0; c < BK; ++c) tr[c] = tv[c];
#pragma unroll
      for (int r = 0; r < B; ++r)
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
          for (int q = 0; q < B; ++q) acc[r * K + k] = fmaf(a[r * B + q], tr[q * K + k], acc[r * K + k]);
    }
  }
#pragma unroll
  for (int c = 0; c < BK; ++c) {
    acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 4);
    acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 2);
    acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 1);
  }
  if (live) {
    const bool own = p_col[s] == agg[i];
    for (int c = g8; c < BK; c += 8) {
      const int r = c / K, k = c % K;
      float v = 0.f;
#pragma unroll
      for (int q = 0; q < B; ++q) {
        float aq = 0.f;
#pragma unroll
        for (int t = 0; t < BK; ++t) aq = t == q * K + k ? acc[t] : aq;
        v = fmaf(dinv[(i * B + r) * B + q], aq, v);
      }
      const float t0 = own ? tval[i * BK + c] : 0.f;
      p_val[s * BK + c] = t0 - omega * v;
    }
  }
}

// A P by contribution lists: block (i, J) of W = A P is the sum over the
// neighbours j of i (ascending) with J in their P row of A_ij P_jJ.  The
// lists (neighbour slot, block of P) are built once with the pattern; here
// a group of 8 lanes sums one block's list with all B x K products in
// registers, then a fixed-order reduction within the group.
template <bool kFill>
__global__ void k_ap_lists(Graph g, const uint8_t* __restrict__ active, const int64_t* __restrict__ p_ptr,
                           const int32_t* __restrict__ p_col, const int64_t* __restrict__ ap_ptr,
                           const int32_t* __restrict__ ap_col, int64_t* __restrict__ cnt, int64_t* __restrict__ cursor,
                           int32_t* __restrict__ cl_k, int32_t* __restrict__ cl_p, int32_t* __restrict__ row) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int64_t a0 = ap_ptr[i];
  const int m = (int)(ap_ptr[i + 1] - a0);
  if (kFill)
    for (int s = 0; s < m; ++s) row[a0 + s] = (int32_t)i;
  if (m == 0 || (active && !active[i])) return;
  const int64_t nb = g.ptr[i];
  const int deg = (int)(g.ptr[i + 1] - nb);
  for (int kk = 0; kk < deg; ++kk) {
    const int32_t j = g.idx[nb + kk];
    for (int64_t pe = p_ptr[j]; pe < p_ptr[j + 1]; ++pe) {
      const int s = bsearch_slot(ap_col + a0, m, p_col[pe]);
      if (s < 0) continue;  // cannot happen: the row is the union of these columns
      if (!kFill) {
        cnt[a0 + s] += 1;
      } else {
        const int64_t pos = cursor[a0 + s]++;
        cl_k[pos] = kk;
        cl_p[pos] = (int32_t)pe;
      }
    }
  }
}

template <int B, int K, bool kSell>
__global__ void __launch_bounds__(256) k_ap_numeric(int64_t n_slots, OpView<B, kSell> A,
                                                    const int64_t* __restrict__ cl_ptr,
                                                    const int32_t* __restrict__ cl_k, const int32_t* __restrict__ cl_p,
                                                    const int32_t* __restrict__ row, const float* __restrict__ p_val,
                                                    float* __restrict__ ap_val) {
  constexpr int BK = B * K;
  const int g8 = threadIdx.x & 7;
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const bool live = s < n_slots;
  float acc[BK];
#pragma unroll
  for (int c = 0; c < BK; ++c) acc[c] = 0.f;
  if (live) {
    const int64_t i = row[s];
    for (int64_t e = cl_ptr[s] + g8; e < cl_ptr[s + 1]; e += 8) {
      const int kk = cl_k[e];
      const float* pv = p_val + (int64_t)cl_p[e] * BK;
      float a[B * B], pr[BK];
#pragma unroll
      for (int c = 0; c < B * B; ++c) a[c] = A.at(i, kk, c);
#pragma unroll
      for (int c = 0; c < BK; ++c) pr[c] = pv[c];
#pragma unroll
      for (int r = 0; r < B; ++r)
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
          for (int q = 0; q < B; ++q) acc[r * K + k] = fmaf(a[r * B + q], pr[q * K + k], acc[r * K + k]);
    }
  }
#pragma unroll
  for (int c = 0; c < BK; ++c) {
    acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 4);
    acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 2);
    acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 1);
  }
  if (live)
    for (int c = g8; c < BK; c += 8) {
      float v = 0.f;
#pragma unroll
      for (int q = 0; q < BK; ++q) v = q == c ? acc[q] : v;
      ap_val[s * BK + c] = v;
    }
}

// Galerkin product A_c = P^T (A P) by contribution lists: every block (I, J)
// of A_c is the sum over the fine rows i of P^T row I (ascending) with J in
// their A P row of P_iI^T W_iJ.  The lists (block of P, block of A P) are
// built once with the pattern; here one warp sums one block's list, a lane
// per contribution with all K x K products in registers, then a fixed-order
// warp reduction.  Decoupled coarse DOFs (a dropped mode: zero row and
// column) get a unit diagonal.
template <bool kFill>
__global__ void k_ac_lists(int64_t n_c, const int64_t* __restrict__ pt_ptr, const int32_t* __restrict__ pt_row,
                           const int64_t* __restrict__ pt_pos, const int64_t* __restrict__ ap_ptr,
                           const int32_t* __restrict__ ap_col, const int64_t* __restrict__ ac_ptr,
                           const int32_t* __restrict__ ac_col, int64_t* __restrict__ cnt,
                           int64_t* __restrict__ cursor, int32_t* __restrict__ cl_p, int32_t* __restrict__ cl_w) {
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n_c) return;
  const int64_t a0 = ac_ptr[I];
  const int m = (int)(ac_ptr[I + 1] - a0);
  for (int64_t pe = pt_ptr[I]; pe < pt_ptr[I + 1]; ++pe) {
    const int32_t i = pt_row[pe];
    for (int64_t ae = ap_ptr[i]; ae < ap_ptr[i + 1]; ++ae) {
      const int s = bsearch_slot(ac_col + a0, m, ap_col[ae]);
      if (s < 0) continue;  // cannot happen: the row is the union of these columns
      if (!kFill) {
        cnt[a0 + s] += 1;
      } else {
        const int64_t pos = cursor[a0 + s]++;
        cl_p[pos] = (int32_t)pt_pos[pe];
        cl_w[pos] = (int32_t)ae;
      }
    }
  }
}

template <int B, int K>
__global__ void __launch_bounds__(256) k_ac_numeric(int64_t n_slots, const int64_t* __restrict__ cl_ptr,
                                                    const int32_t* __restrict__ cl_p, const int32_t* __restrict__ cl_w,
                                                    const float* __restrict__ p_val, const float* __restrict__ ap_val,
                                                    const int32_t* __restrict__ slot_row,
                                                    const int32_t* __restrict__ ac_col, float* __restrict__ ac_val) {
  constexpr int BK = B * K, KK = K * K;
  const int lane = threadIdx.x & 31;
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= n_slots) return;
  float acc[KK];
#pragma unroll
  for (int c = 0; c < KK; ++c) acc[c] = 0.f;
  for (int64_t e = cl_ptr[s] + lane; e < cl_ptr[s + 1]; e += 32) {
    const float* pv = p_val + (int64_t)cl_p[e] * BK;
    const float* wv = ap_val + (int64_t)cl_w[e] * BK;
    float pr[BK], wr[BK];
#pragma unroll
    for (int c = 0; c < BK; ++c) {
      pr[c] = pv[c];
      wr[c] = wv[c];
    }
#pragma unroll
    for (int k1 = 0; k1 < K; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < K; ++k2)
#pragma unroll
        for (int q = 0; q < B; ++q) acc[k1 * K + k2] = fmaf(pr[q * K + k1], wr[q * K + k2], acc[k1 * K + k2]);
  }
#pragma unroll
  for (int c = 0; c < KK; ++c) acc[c] = warp_sum(acc[c]);
  const bool diag = ac_col[s] == slot_row[s];
  for (int c = lane; c < KK; c += 32) {
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < KK; ++q) v = q == c ? acc[q] : v;
    if (diag && c / K == c % K && v == 0.f) v = 1.f;
    ac_val[s * KK + c] = v;
  }
}

// Row of every block slot of a block CSR pattern.
__global__ void k_slot_rows(int64_t n, const int64_t* __restrict__ ptr, int32_t* __restrict__ row) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) row[e] = (int32_t)i;
}

// Inverse of the diagonal block of every coarse row (Gauss-Jordan, partial
// pivoting, FP64).
template <int K>
__global__ void k_block_inv(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ col,
                            const float* __restrict__ val, float* __restrict__ dinv, int32_t* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t d = -1;
  for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e)
    if (col[e] == (int32_t)i) d = e;
  double M[K][2 * K];
  for (int p = 0; p < K; ++p)
    for (int q = 0; q < K; ++q) {
      M[p][q] = d >= 0 ? (double)val[d * K * K + p * K + q] : 0.0;
      M[p][K + q] = p == q ? 1.0 : 0.0;
    }
  bool ok = d >= 0;
  for (int c = 0; c < K && ok; ++c) {
    int piv = c;
    for (int p = c + 1; p < K; ++p)
      if (fabs(M[p][c]) > fabs(M[piv][c])) piv = p;
    if (!(fabs(M[piv][c]) > 0.0)) {
      ok = false;
      break;
    }
    if (piv != c)
      for (int q = 0; q < 2 * K; ++q) {
        const double t = M[c][q];
        M[c][q] = M[piv][q];
        M[piv][q] = t;
      }
    const double inv = 1.0 / M[c][c];
    for (int q = 0; q < 2 * K; ++q) M[c][q] *= inv;
    for (int p = 0; p < K; ++p)
      if (p != c) {
        const double f = M[p][c];
        for (int q = 0; q < 2 * K; ++q) M[p][q] -= f * M[c][q];
      }
  }
  if (!ok) flag_status(status, kStatNonFinite);
  for (int p = 0; p < K; ++p)
    for (int q = 0; q < K; ++q) dinv[(i * K + p) * K + q] = ok ? (float)M[p][K + q] : 0.f;
}

// Dense inverse of the coarsest operator (m <= kCoarseMaxDof), one CTA,
// Gauss-Jordan with partial pivoting in FP64 on [A | I] held in `work`
// (m x 2m), symmetrised on output.
__global__ void __launch_bounds__(1024) k_coarse_inverse(int64_t n, int K, const int64_t* __restrict__ ptr,
                                                         const int32_t* __restrict__ col,
                                                         const float* __restrict__ val, double* __restrict__ work,
                                                         float* __restrict__ inv, int32_t* __restrict__ status) {
  __shared__ int piv_s;
  __shared__ bool ok_s;
  __shared__ double fcol[kCoarseMaxDof];
  const int m = (int)(n * K);
  const int w2 = 2 * m;
  for (int t = threadIdx.x; t < m * w2; t += blockDim.x) work[t] = (t % w2) - m == t / w2 ? 1.0 : 0.0;
  __syncthreads();
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e)
      for (int p = 0; p < K; ++p)
        for (int q = 0; q < K; ++q) work[(i * K + p) * w2 + (int64_t)col[e] * K + q] = val[e * K * K + p * K + q];
  if (threadIdx.x == 0) ok_s = true;
  __syncthreads();
  for (int c = 0; c < m; ++c) {
    if (threadIdx.x == 0) {
      int piv = c;
      for (int p = c + 1; p < m; ++p)
        if (fabs(work[p * w2 + c]) > fabs(work[piv * w2 + c])) piv = p;
      if (!(fabs(work[piv * w2 + c]) > 0.0)) ok_s = false;
      piv_s = piv;
    }
    __syncthreads();
    if (!ok_s) break;
    const int piv = piv_s;
    if (piv != c)
      for (int q = threadIdx.x; q < w2; q += blockDim.x) {
        const double t = work[c * w2 + q];
        work[c * w2 + q] = work[piv * w2 + q];
        work[piv * w2 + q] = t;
      }
    __syncthreads();
    const double inv_p = 1.0 / work[c * w2 + c];
    __syncthreads();
    for (int q = threadIdx.x; q < w2; q += blockDim.x) work[c * w2 + q] *= inv_p;
    __syncthreads();
    // multipliers first: the elimination below overwrites column c
    for (int p = threadIdx.x; p < m; p += blockDim.x) fcol[p] = p == c ? 0.0 : work[p * w2 + c];
    __syncthreads();
    for (int t = threadIdx.x; t < m * w2; t += blockDim.x) {
      const int p = t / w2, q = t % w2;
      if (p != c) work[t] -= fcol[p] * work[c * w2 + q];
    }
    __syncthreads();
  }
  if (!ok_s) {
    if (threadIdx.x == 0) flag_status(status, kStatNonFinite);
    return;
  }
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int p = t / m, q = t % m;
    inv[t] = (float)(0.5 * (work[p * w2 + m + q] + work[q * w2 + m + p]));
  }
}

// ================================================================== solve ==
enum { kOpS1 = 1, kOpS2, kOpS3, kOpS4, kOpS4Dot, kOpQ, kOpLzQ, kOpQc };

// Level vectors of the V-cycle and the CG scalars the fused kernels touch.
struct OpArgs {
  float* f;        // right-hand side of the level
  float* x;        // pre-smoothed iterate
  float* xb;       // post-smoothed iterate (the level's output)
  float* r;        // residual
  float* d;        // Chebyshev directions (two buffers: the SpMV operand is never written)
  float* db;
  const float* dinv;
  float theta_inv, c1, c2;
  float* p;        // kOpQ / kOpLzQ operand; kOpQc updates it
  float* q;
  double* partial;
  AmgCtrl* ctrl;
  double* lz;      // Lanczos coefficients (kOpLzQ)
  const __half* sv16;    // level 0: FP16 smoothing copy of the sliced matrix (scaled by 1 / *s16inv)
  const float* s16inv;
};

template <int MODE>
__device__ __forceinline__ const float* op_operand(const OpArgs& a) {
  if constexpr (MODE == kOpS1 || MODE == kOpS4 || MODE == kOpS4Dot) return a.d;
  else if constexpr (MODE == kOpS2) return a.db;
  else if constexpr (MODE == kOpS3) return a.x;
  else if constexpr (MODE == kOpQc) return a.xb;  // z, the preconditioned residual
  else return a.p;
}

// Row epilogue shared by the sliced and CSR kernels: y = (A v)_i; returns the
// row's contribution to the kernel's dot product.
template <int B, int MODE>
__device__ __forceinline__ double op_epilogue(const OpArgs& a, int64_t i, const float (&y)[B]) {
  const int64_t o = i * B;
  float t[B], rn[B];
  double dot = 0.0;
  if constexpr (MODE == kOpS1) {
#pragma unroll
    for (int c = 0; c < B; ++c) rn[c] = a.f[o + c] - y[c];
    block_mv<B>(a.dinv + i * B * B, rn, t);
#pragma unroll
    for (int c = 0; c < B; ++c) {
      const float dn = a.c1 * a.d[o + c] + a.c2 * t[c];
      a.r[o + c] = rn[c];
      a.db[o + c] = dn;
      a.x[o + c] += dn;
    }
  } else if constexpr (MODE == kOpS2) {
#pragma unroll
    for (int c = 0; c < B; ++c) a.r[o + c] -= y[c];
  } else if constexpr (MODE == kOpS3) {
#pragma unroll
    for (int c = 0; c < B; ++c) rn[c] = a.f[o + c] - y[c];
    block_mv<B>(a.dinv + i * B * B, rn, t);
#pragma unroll
    for (int c = 0; c < B; ++c) {
      const float dn = a.theta_inv * t[c];
      a.r[o + c] = rn[c];
      a.d[o + c] = dn;
      a.xb[o + c] = a.x[o + c] + dn;
    }
  } else if constexpr (MODE == kOpS4 || MODE == kOpS4Dot) {
#pragma unroll
    for (int c = 0; c < B; ++c) rn[c] = a.r[o + c] - y[c];
    block_mv<B>(a.dinv + i * B * B, rn, t);
#pragma unroll
    for (int c = 0; c < B; ++c) {
      const float z = a.xb[o + c] + (a.c1 * a.d[o + c] + a.c2 * t[c]);
      a.xb[o + c] = z;
      if constexpr (MODE == kOpS4Dot) dot += (double)a.f[o + c] * (double)z;
    }
  } else if constexpr (MODE == kOpQc) {
    // direction update folded into the product: p = z + beta p and
    // q = A z + beta q, which carries A p by recurrence between restarts
    const float beta = (float)a.ctrl->beta;
#pragma unroll
    for (int c = 0; c < B; ++c) {
      const float pn = a.xb[o + c] + beta * a.p[o + c];
      const float qn = y[c] + beta * a.q[o + c];
      a.p[o + c] = pn;
      a.q[o + c] = qn;
      dot += (double)pn * (double)qn;
    }
  } else {
#pragma unroll
    for (int c = 0; c < B; ++c) {
      a.q[o + c] = y[c];
      dot += (double)a.p[o + c] * (double)y[c];
    }
  }
  return dot;
}

// Only an exact zero or a non-finite value stops the iteration, as in the
// block-Jacobi CG and the reference's CG: a Neo-Hookean tangent under large
// deformation can be mildly indefinite, and CG usually converges through a
// negative curvature p.Ap or r.z on it.
template <int MODE>
__device__ __forceinline__ void op_finish(const OpArgs& a, double tot) {
  AmgCtrl* c = a.ctrl;
  if constexpr (MODE == kOpS4Dot) {
    if (!isfinite(tot)) c->done = kNonFinite;
    else if (tot == 0.0) c->done = kBreakdown;
    else {
      c->beta = tot / c->rz * c->pscale;
      c->rz = tot;
      c->pscale = 1.0;
    }
  } else if constexpr (MODE == kOpQ || MODE == kOpLzQ || MODE == kOpQc) {
    if (!isfinite(tot)) c->done = kNonFinite;
    else if (tot == 0.0 || (MODE == kOpLzQ && tot < 0.0)) c->done = kBreakdown;
    else {
      c->alpha = c->rz / tot;
      if constexpr (MODE == kOpLzQ) a.lz[2 * c->lz_step] = c->alpha;
    }
  }
}

template <int MODE>
__host__ __device__ constexpr bool op_has_dot() {
  return MODE == kOpS4Dot || MODE == kOpQ || MODE == kOpLzQ || MODE == kOpQc;
}

// Level 0: the sliced FP32 matrix (the layout of fem_assemble_sell): one CTA
// per slice of 32 rows, thread per row, the kSellW warps sharing the slice's
// slots (short dependent chains), partial rows summed in shared memory in a
// fixed order.  The grid covers every slice, so the hardware balances the
// tail.  The matrix streams with L2 evict_first; the vectors stay in L2.
//
// The smoothing passes (S1..S4) may read an FP16 copy of the same matrix
// instead (sv16, built by k_sell_to_half): Chebyshev smoothing only has to
// damp the rough error, and one consistent copy in all four passes keeps the
// V-cycle a fixed symmetric operator (pre- and post-smoothing are adjoint),
// so CG still applies; CG's own q = A p always uses the FP32 matrix.
__device__ __forceinline__ uint32_t ld_l2_b32(const void* ptr, uint64_t pol) {
  uint32_t v;
  asm("ld.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(ptr), "l"(pol));
  return v;
}

__device__ __forceinline__ uint16_t ld_l2_b16(const void* ptr, uint64_t pol) {
  uint16_t v;
  asm("ld.global.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(ptr), "l"(pol));
  return v;
}

// The DD values of slot-row entry `lane` of the FP16 copy.  Layout of one
// slot-row (32 rows, DD values each, DD * 64 bytes): the value pairs (0,1),
// (2,3), ... as [pair][lane] half2 words, then an odd last value as [lane]
// halves.  base16 points at the slot-row.
template <int DD>
__device__ __forceinline__ void load_slot16(const __half* __restrict__ base16, int lane, uint64_t pol,
                                            float (&m)[DD]) {
#pragma unroll
  for (int p = 0; p < DD / 2; ++p) {
    const uint32_t w = ld_l2_b32(base16 + p * 64 + 2 * lane, pol);
    const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w));
    m[2 * p] = f.x;
    m[2 * p + 1] = f.y;
  }
  if constexpr (DD % 2 == 1) {
    const uint16_t hv = ld_l2_b16(base16 + (DD / 2) * 64 + lane, pol);
    m[DD - 1] = __half2float(*reinterpret_cast<const __half*>(&hv));
  }
}

// The smoothing modes, which may read the FP16 copy.
template <int MODE>
__host__ __device__ constexpr bool op_smoothing() {
  return MODE == kOpS1 || MODE == kOpS2 || MODE == kOpS3 || MODE == kOpS4 || MODE == kOpS4Dot;
}

// Values of slot k of this thread's row: FP32 matrix, or the FP16 copy (H).
template <int DD, bool H>
__device__ __forceinline__ void load_slot(const float* __restrict__ vp, const __half* __restrict__ hp, int k,
                                          int lane, uint64_t pol, float (&m)[DD]) {
  if constexpr (H) {
    load_slot16<DD>(hp + (int64_t)k * DD * 32, lane, pol, m);
  } else {
    const float* vk = vp + (int64_t)k * DD * 32;
#pragma unroll
    for (int e = 0; e < DD; ++e) m[e] = ld_l2(vk + e * 32, pol);
  }
}

template <int D, int MODE, bool H>
__global__ void __launch_bounds__(kSellW * 32) k_sell_op(int64_t n_rows, const int64_t* __restrict__ sell_base,
                                                         const int32_t* __restrict__ col,
                                                         const float* __restrict__ sval, OpArgs a) {
  constexpr int DD = D * D;
  __shared__ float ys[kSellW][D][32];
  pdl_enter();
  if (amg_idle(a.ctrl)) return;
  const float* __restrict__ v = op_operand<MODE>(a);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t pol = l2_policy(false);
  double dot = 0.0;
  const int64_t s = blockIdx.x;
  const int64_t b0 = sell_base[s];
  const int len = (int)((sell_base[s + 1] - b0) >> 5);
  const int32_t* cp = col + b0 + lane;
  const float* vp = sval + b0 * DD + lane;
  const __half* hp = H ? a.sv16 + b0 * DD : nullptr;
  float y[D];
#pragma unroll
  for (int c = 0; c < D; ++c) y[c] = 0.f;
  static_assert(D > 1, "scalar rows use k_sell_op1");
#pragma unroll 2
  for (int k = w; k < len; k += kSellW) {
    const int64_t cc = ld_l2(cp + (int64_t)k * 32, pol);
    float m[DD];
    load_slot<DD, H>(vp, hp, k, lane, pol, m);
    float xv[D];
#pragma unroll
    for (int j = 0; j < D; ++j) xv[j] = v[cc * D + j];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int j = 0; j < D; ++j) y[r] = fmaf(m[r * D + j], xv[j], y[r]);
  }
#pragma unroll
  for (int c = 0; c < D; ++c) ys[w][c][lane] = y[c];
  __syncthreads();
  if (w == 0) {
    const int64_t i = s * 32 + lane;
    if (i < n_rows) {
      const float sc = H ? *a.s16inv : 1.f;  // a power of two: exact
      float yt[D];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        float t = ys[0][c][lane];
#pragma unroll
        for (int u = 1; u < kSellW; ++u) t += ys[u][c][lane];
        yt[c] = H ? t * sc : t;
      }
      dot += op_epilogue<D, MODE>(a, i, yt);
    }
  }
  // the modes that end in a dot product leave the slice's share of it in
  // partial[slice]; k_dot_finish adds them (no CTA waits on another, and
  // warps 1-3 are done as soon as their rows are in shared memory)
  if constexpr (op_has_dot<MODE>()) {
    if (w == 0) {
      const double t = warp_sum(dot);
      if (lane == 0) a.partial[blockIdx.x] = t;
    }
  }
}

// Level 0 with the slice streamed by bulk copies (cp.async.bulk): one CTA per
// slice as in k_sell_op, but thread 0 copies the slice's slot-rows (values
// and columns) into a two-stage shared-memory ring, kTma0Rows slot-rows a
// stage, completing on an mbarrier per stage; the warps read their slot-rows
// from shared memory and gather x from L2.  A few bulk copies per CTA keep
// more bytes in flight than one slot's loads per thread.  Every stage wait is
// bounded (kTma0Spin cycles): on a timeout the CTA flags kBarrierTimeout,
// waits (bounded) for the copies it issued and returns.
#ifndef TFG_TMA0_ROWS
#define TFG_TMA0_ROWS 8
#endif
constexpr int kTma0Rows = TFG_TMA0_ROWS;  // slot-rows per ring stage
constexpr long long kTma0Spin = 2000000000LL;

template <int D, bool H>
__host__ __device__ constexpr int tma0_vbytes() { return H ? D * D * 64 : D * D * 128; }  // per slot-row
template <int D, bool H>
__host__ __device__ constexpr int tma0_stage() { return kTma0Rows * (tma0_vbytes<D, H>() + 128); }

__device__ __forceinline__ uint32_t amg_smem_u32(const void* ptr) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ bool amg_mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kTma0Spin) return false;
  }
}

// Stage c of the slice: its slot-rows' values then columns (16-byte aligned:
// slices start at multiples of 32 slots).
template <int D, bool H>
__device__ __forceinline__ void tma0_issue(uint32_t bar, uint32_t dst, const void* vals, const int32_t* cols,
                                           int nr, uint64_t pol) {
  const uint32_t vb = (uint32_t)(nr * tma0_vbytes<D, H>()), cb = (uint32_t)(nr * 128);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(vb + cb) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst),
      "l"(vals), "r"(vb), "r"(bar), "l"(pol)
      : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          dst + (uint32_t)(kTma0Rows * tma0_vbytes<D, H>())),
      "l"(cols), "r"(cb), "r"(bar), "l"(pol)
      : "memory");
}

template <int D, int MODE, bool H>
__global__ void __launch_bounds__(kSellW * 32) k_sell_op_tma(int64_t n_rows, const int64_t* __restrict__ sell_base,
                                                             const int32_t* __restrict__ col,
                                                             const float* __restrict__ sval, OpArgs a) {
  constexpr int DD = D * D;
  constexpr int VB = tma0_vbytes<D, H>();
  constexpr int SB = tma0_stage<D, H>();
  extern __shared__ __align__(128) unsigned char ring[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ float ys[kSellW][D][32];
  pdl_enter();
  if (amg_idle(a.ctrl)) return;
  const float* __restrict__ v = op_operand<MODE>(a);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t pol = l2_policy(false);
  const int64_t s = blockIdx.x;
  const int64_t b0 = sell_base[s];
  const int len = (int)((sell_base[s + 1] - b0) >> 5);
  const int nch = (len + kTma0Rows - 1) / kTma0Rows;
  const uint32_t bar0 = amg_smem_u32(&bars[0]), buf0 = amg_smem_u32(ring);
  const char* vsrc = H ? reinterpret_cast<const char*>(a.sv16 + b0 * DD) : reinterpret_cast<const char*>(sval + b0 * DD);
  auto issue = [&](int c) {
    const int r0 = c * kTma0Rows;
    tma0_issue<D, H>(bar0 + 8u * (uint32_t)(c & 1), buf0 + (uint32_t)((c & 1) * SB), vsrc + (int64_t)r0 * VB,
                     col + b0 + (int64_t)r0 * 32, min(kTma0Rows, len - r0), pol);
  };
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int c = 0; c < 2 && c < nch; ++c) issue(c);
  }
  __syncthreads();
  float y[D];
#pragma unroll
  for (int c = 0; c < D; ++c) y[c] = 0.f;
  int done = 0;  // stages consumed
  bool ok = true;
  for (int c = 0; c < nch; ++c) {
    const bool got = amg_mbar_wait(bar0 + 8u * (uint32_t)(c & 1), (uint32_t)((c >> 1) & 1));
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    const unsigned char* st = ring + (c & 1) * SB;
    const int32_t* cs = reinterpret_cast<const int32_t*>(st + kTma0Rows * VB);
    const int nr = min(kTma0Rows, len - c * kTma0Rows);
    for (int k = w; k < nr; k += kSellW) {
      const int64_t cc = cs[k * 32 + lane];
      float m[DD];
      if constexpr (H) {
        const uint32_t* wv = reinterpret_cast<const uint32_t*>(st + k * VB);
#pragma unroll
        for (int p = 0; p < DD / 2; ++p) {
          const uint32_t wd = wv[p * 32 + lane];
          const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&wd));
          m[2 * p] = f.x;
          m[2 * p + 1] = f.y;
        }
        if constexpr (DD % 2 == 1) {
          const __half* hv = reinterpret_cast<const __half*>(st + k * VB) + (DD / 2) * 64;
          m[DD - 1] = __half2float(hv[lane]);
        }
      } else {
        const float* fv = reinterpret_cast<const float*>(st + k * VB);
#pragma unroll
        for (int e = 0; e < DD; ++e) m[e] = fv[e * 32 + lane];
      }
      float xv[D];
#pragma unroll
      for (int j = 0; j < D; ++j) xv[j] = v[cc * D + j];
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int j = 0; j < D; ++j) y[r] = fmaf(m[r * D + j], xv[j], y[r]);
    }
    done = c + 1;
    __syncthreads();  // every warp is done with this stage
    if (threadIdx.x == 0 && c + 2 < nch) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(c + 2);
    }
  }
  if (!ok) {
    // flag, then wait (bounded) for this CTA's copies still in flight
    if (threadIdx.x == 0) {
      atomicExch(&a.ctrl->done, kBarrierTimeout);
      const int issued = min(nch, done + 2);
      for (int c = done; c < issued; ++c) amg_mbar_wait(bar0 + 8u * (uint32_t)(c & 1), (uint32_t)((c >> 1) & 1));
    }
    __syncthreads();
    return;
  }
#pragma unroll
  for (int c = 0; c < D; ++c) ys[w][c][lane] = y[c];
  __syncthreads();
  double dot = 0.0;
  if (w == 0) {
    const int64_t i = s * 32 + lane;
    if (i < n_rows) {
      const float sc = H ? *a.s16inv : 1.f;  // a power of two: exact
      float yt[D];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        float t = ys[0][c][lane];
#pragma unroll
        for (int u = 1; u < kSellW; ++u) t += ys[u][c][lane];
        yt[c] = H ? t * sc : t;
      }
      dot += op_epilogue<D, MODE>(a, i, yt);
    }
  }
  if constexpr (op_has_dot<MODE>()) {
    if (w == 0) {
      const double t = warp_sum(dot);
      if (lane == 0) a.partial[blockIdx.x] = t;
    }
  }
}

// Level 0 of a scalar field (heat): a slot holds one 4-byte value, so a
// 32-row slice is only a few KB and the shared-slot CTA of k_sell_op spends
// more on its CTA and its shared-memory sum than on streaming.  Here each warp
// owns one slice (kSell1W slices per CTA), each thread its row, and a thread
// walks all of the row's slots in batches of kSell1U: the next batch's
// column and value loads are issued before the current batch's gathers, so
// the matrix stream never waits on the vector gathers.  No shared memory, no
// barrier; the slots are summed in order.  Per-slice dot shares as in
// k_sell_op, so k_dot_finish is the same.
constexpr int kSell1W = 4;
constexpr int kSell1U = 4;

// Columns and values of slots k .. k + kSell1U - 1 of this thread's row (the
// slots at or past len are not read and contribute 0 at column 0).
template <bool H>
__device__ __forceinline__ void sell1_batch(const int32_t* __restrict__ cp, const float* __restrict__ vp,
                                            const __half* __restrict__ hp, int k, int len, int lane,
                                            uint64_t pol, int32_t (&c)[kSell1U], float (&m)[kSell1U]) {
#pragma unroll
  for (int u = 0; u < kSell1U; ++u) {
    c[u] = 0;
    m[u] = 0.f;
    if (k + u < len) {
      float t[1];
      c[u] = ld_l2(cp + (int64_t)(k + u) * 32, pol);
      load_slot<1, H>(vp, hp, k + u, lane, pol, t);
      m[u] = t[0];
    }
  }
}

template <int MODE, bool H>
__global__ void __launch_bounds__(kSell1W * 32) k_sell_op1(int64_t n_rows, int64_t n_slices,
                                                           const int64_t* __restrict__ sell_base,
                                                           const int32_t* __restrict__ col,
                                                           const float* __restrict__ sval, OpArgs a) {
  pdl_enter();
  if (amg_idle(a.ctrl)) return;
  const int lane = threadIdx.x & 31;
  const int64_t s = (int64_t)blockIdx.x * kSell1W + (threadIdx.x >> 5);
  if (s >= n_slices) return;
  const float* __restrict__ v = op_operand<MODE>(a);
  const uint64_t pol = l2_policy(false);
  const int64_t b0 = sell_base[s];
  const int len = (int)((sell_base[s + 1] - b0) >> 5);
  const int32_t* cp = col + b0 + lane;
  const float* vp = sval + b0 + lane;
  const __half* hp = H ? a.sv16 + b0 : nullptr;
  float y = 0.f;
  int32_t cc[kSell1U];
  float mv[kSell1U];
  sell1_batch<H>(cp, vp, hp, 0, len, lane, pol, cc, mv);
  for (int k = 0; k < len; k += kSell1U) {
    int32_t cn[kSell1U];
    float mn[kSell1U];
    sell1_batch<H>(cp, vp, hp, k + kSell1U, len, lane, pol, cn, mn);
#pragma unroll
    for (int u = 0; u < kSell1U; ++u)
      if (k + u < len) y = fmaf(mv[u], v[cc[u]], y);
#pragma unroll
    for (int u = 0; u < kSell1U; ++u) {
      cc[u] = cn[u];
      mv[u] = mn[u];
    }
  }
  double dot = 0.0;
  const int64_t i = s * 32 + lane;
  if (i < n_rows) {
    const float yt[1] = {H ? y * *a.s16inv : y};  // a power of two: exact
    dot = op_epilogue<1, MODE>(a, i, yt);
  }
  if constexpr (op_has_dot<MODE>()) {
    const double t = warp_sum(dot);
    if (lane == 0) a.partial[s] = t;
  }
}

// The scalar kernel with each warp's slice staged by bulk copies: lane 0
// copies the slice's values and columns (contiguous, slot-major) into the
// warp's part of shared memory with two cp.async.bulk on one mbarrier, then
// the warp reads them from there; the same sums in the same order as
// k_sell_op1.  Slices longer than kSell1Max slot-rows load directly.  The
// wait is bounded: on a timeout the warp flags kBarrierTimeout, waits once
// more (bounded) for its copy and returns.
constexpr int kSell1Max = 32;

template <bool H>
__host__ __device__ constexpr int sell1_vb() { return H ? 64 : 128; }  // value bytes per slot-row
template <bool H>
__host__ __device__ constexpr int sell1_smem() { return kSell1W * kSell1Max * (sell1_vb<H>() + 128); }

template <int MODE, bool H>
__global__ void __launch_bounds__(kSell1W * 32) k_sell_op1_tma(int64_t n_rows, int64_t n_slices,
                                                               const int64_t* __restrict__ sell_base,
                                                               const int32_t* __restrict__ col,
                                                               const float* __restrict__ sval, OpArgs a) {
  constexpr int VB = sell1_vb<H>();
  extern __shared__ __align__(128) unsigned char ring[];
  __shared__ __align__(8) uint64_t bars[kSell1W];
  pdl_enter();
  if (amg_idle(a.ctrl)) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t s = (int64_t)blockIdx.x * kSell1W + w;
  if (s >= n_slices) return;
  const float* __restrict__ v = op_operand<MODE>(a);
  const uint64_t pol = l2_policy(false);
  const int64_t b0 = sell_base[s];
  const int len = (int)((sell_base[s + 1] - b0) >> 5);
  float y = 0.f;
  if (len <= kSell1Max) {
    unsigned char* wbuf = ring + (size_t)w * kSell1Max * (VB + 128);
    const uint32_t bar = amg_smem_u32(&bars[w]), dst = amg_smem_u32(wbuf);
    if (lane == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      if (len > 0) {
        const uint32_t vb = (uint32_t)(len * VB), cb = (uint32_t)(len * 128);
        const void* vsrc = H ? (const void*)(a.sv16 + b0) : (const void*)(sval + b0);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(vb + cb) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
            "%4;" ::"r"(dst),
            "l"(vsrc), "r"(vb), "r"(bar), "l"(pol)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
            "%4;" ::"r"(dst + (uint32_t)(kSell1Max * VB)),
            "l"(col + b0), "r"(cb), "r"(bar), "l"(pol)
            : "memory");
      }
    }
    __syncwarp();
    const bool got = len == 0 || amg_mbar_wait(bar, 0);
    if (!__all_sync(0xffffffffu, got)) {
      if (lane == 0) {
        atomicExch(&a.ctrl->done, kBarrierTimeout);
        amg_mbar_wait(bar, 0);
      }
      __syncwarp();
      return;
    }
    const int32_t* cs = reinterpret_cast<const int32_t*>(wbuf + kSell1Max * VB);
    int k = 0;
    for (; k + 4 <= len; k += 4) {
      float m[4], xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int kk = k + u;
        m[u] = H ? __half2float(reinterpret_cast<const __half*>(wbuf)[kk * 32 + lane])
                 : reinterpret_cast<const float*>(wbuf)[kk * 32 + lane];
        xv[u] = v[cs[kk * 32 + lane]];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) y = fmaf(m[u], xv[u], y);
    }
    for (; k < len; ++k) {
      const float m = H ? __half2float(reinterpret_cast<const __half*>(wbuf)[k * 32 + lane])
                        : reinterpret_cast<const float*>(wbuf)[k * 32 + lane];
      y = fmaf(m, v[cs[k * 32 + lane]], y);
    }
  } else {
    const int32_t* cp = col + b0 + lane;
    const float* vp = sval + b0 + lane;
    const __half* hp = H ? a.sv16 + b0 : nullptr;
    int32_t cc[kSell1U];
    float mv[kSell1U];
    sell1_batch<H>(cp, vp, hp, 0, len, lane, pol, cc, mv);
    for (int k = 0; k < len; k += kSell1U) {
      int32_t cn[kSell1U];
      float mn[kSell1U];
      sell1_batch<H>(cp, vp, hp, k + kSell1U, len, lane, pol, cn, mn);
#pragma unroll
      for (int u = 0; u < kSell1U; ++u)
        if (k + u < len) y = fmaf(mv[u], v[cc[u]], y);
#pragma unroll
      for (int u = 0; u < kSell1U; ++u) {
        cc[u] = cn[u];
        mv[u] = mn[u];
      }
    }
  }
  double dot = 0.0;
  const int64_t i = s * 32 + lane;
  if (i < n_rows) {
    const float yt[1] = {H ? y * *a.s16inv : y};  // a power of two: exact
    dot = op_epilogue<1, MODE>(a, i, yt);
  }
  if constexpr (op_has_dot<MODE>()) {
    const double t = warp_sum(dot);
    if (lane == 0) a.partial[s] = t;
  }
}

// A launch of the CG iteration's kernel chain: with g_amg_pdl, through
// cudaLaunchKernelEx with programmatic stream serialization (the kernel's
// pdl_enter waits for its predecessor).
template <typename... Ex, typename... Act>
void launch_chain(dim3 g, dim3 b, size_t smem, cudaStream_t st, void (*k)(Ex...), Act&&... args) {
  if (!g_amg_pdl) {
    k<<<g, b, smem, st>>>(std::forward<Act>(args)...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = g;
  cfg.blockDim = b;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, std::forward<Act>(args)...);
}

// One level-0 pass: the shared-slot kernel for 2×2 / 3×3 blocks, the
// warp-per-slice kernel for scalar rows.
template <int D, int MODE, bool H>
void launch_sell(int64_t n, const int64_t* sell_base, const int32_t* sell_col, const float* sell_val,
                 const OpArgs& a, cudaStream_t st) {
  const int64_t ns = (n + 31) / 32;
  if constexpr (D == 1) {
    const unsigned g = (unsigned)((ns + kSell1W - 1) / kSell1W);
    if (g_amg_tma)
      launch_chain(g, kSell1W * 32, sell1_smem<H>(), st, k_sell_op1_tma<MODE, H>, n, ns, sell_base, sell_col,
                   sell_val, a);
    else
      launch_chain(g, kSell1W * 32, 0, st, k_sell_op1<MODE, H>, n, ns, sell_base, sell_col, sell_val, a);
  } else if (g_amg_tma) {
    launch_chain((unsigned)ns, kSellW * 32, 2 * tma0_stage<D, H>(), st, k_sell_op_tma<D, MODE, H>, n, sell_base,
                 sell_col, sell_val, a);
  } else {
    launch_chain((unsigned)ns, kSellW * 32, 0, st, k_sell_op<D, MODE, H>, n, sell_base, sell_col, sell_val, a);
  }
}

// The dot product of a level-0 pass that ends in one: the per-slice shares
// left by k_sell_op added in a fixed order by one CTA, then the CG (or
// Lanczos) scalar update.  Deterministic; idle exactly when the pass was.
template <int MODE>
__global__ void __launch_bounds__(1024) k_dot_finish(int64_t n, OpArgs a) {
  __shared__ double red[32];
  pdl_enter();
  if (amg_idle(a.ctrl)) return;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(a.partial + i);
  const double tot = block_sum(s, red);
  if (threadIdx.x == 0) op_finish<MODE>(a, tot);
}

// The FP16 smoothing copy: max |a_ij| over the sliced FP32 values (as the
// bit pattern of a non-negative float, whose integer order is the float
// order; a max is exact and order-independent).
__global__ void k_abs_max(int64_t n, const float* __restrict__ v, unsigned int* __restrict__ out) {
  float m = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(v[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// Power-of-two scale that maps max |a_ij| into [2^13, 2^14): every value
// keeps FP16's 11-bit significand down to 2^-24 of the largest one, far from
// FP16's maximum 65504.
__device__ __forceinline__ float half_scale(unsigned int maxbits, bool inverse) {
  const float mx = __uint_as_float(maxbits);
  if (!(mx > 0.f) || !isfinite(mx)) return 1.f;
  int e;
  frexpf(mx, &e);
  return ldexpf(1.f, inverse ? e - 14 : 14 - e);
}

// FP16 copy of the sliced matrix in the slot-row layout of load_slot16, a
// thread per (slot-row, row).
template <int DD>
__global__ void k_sell_to_half(int64_t n_blocks, const float* __restrict__ sval,
                               const unsigned int* __restrict__ maxbits, __half* __restrict__ sv16,
                               float* __restrict__ s16inv) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) *s16inv = half_scale(*maxbits, true);
  if (t >= n_blocks) return;
  const float sc = half_scale(*maxbits, false);
  const int64_t sr = t >> 5;
  const int lane = (int)(t & 31);
  const float* src = sval + sr * 32 * DD + lane;
  __half* dst = sv16 + sr * 32 * DD;
#pragma unroll
  for (int e = 0; e < DD; ++e) {
    const __half hv = __float2half_rn(src[e * 32] * sc);
    if (DD % 2 == 1 && e == DD - 1) dst[(DD / 2) * 64 + lane] = hv;
    else dst[(e / 2) * 64 + 2 * lane + (e & 1)] = hv;
  }
}

// Coarser levels: block CSR (B x B blocks), one CTA of 128 threads per row;
// thread t < 120 takes row t % B of every (120 / B)-th block, so every
// thread keeps one component and the per-component sums run in a fixed
// order.  The epilogue runs on threads t < B.  Coarse operators are read
// evict_last so they stay in L2 across the cycle.
constexpr int kRowT = 128;   // threads per coarse row
constexpr int kRowItems = 120;  // of which hold (block, component) items: a multiple of 2, 3 and 6

template <int B, int MODE>
__global__ void __launch_bounds__(kRowT) k_csr_op(int64_t n, const int64_t* __restrict__ ptr,
                                                  const int32_t* __restrict__ col, const float* __restrict__ val,
                                                  OpArgs a) {
  constexpr int PB = kRowItems / B;
  __shared__ float part[kRowItems];
  __shared__ float rs[B];
  __shared__ double red[32];
  if (amg_idle(a.ctrl)) return;
  const float* __restrict__ v = op_operand<MODE>(a);
  const int t = threadIdx.x;
  const int r = t % B, u = t / B;
  const uint64_t pol = l2_policy(true);
  double dot = 0.0;
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    if (t < kRowItems) {
      constexpr int U = 4;  // passes whose loads are in flight together
      float y = 0.f;
      const int64_t e1 = ptr[i + 1];
      for (int64_t e = ptr[i] + u; e < e1; e += U * PB) {
        int64_t c[U];
#pragma unroll
        for (int w = 0; w < U; ++w) c[w] = e + w * PB < e1 ? (int64_t)ld_l2(col + e + w * PB, pol) : -1;
        float m[U][B], xv[U][B];
#pragma unroll
        for (int w = 0; w < U; ++w)
#pragma unroll
          for (int q = 0; q < B; ++q) {
            m[w][q] = c[w] >= 0 ? ld_l2(val + (e + w * PB) * B * B + r * B + q, pol) : 0.f;
            xv[w][q] = c[w] >= 0 ? v[c[w] * B + q] : 0.f;
          }
#pragma unroll
        for (int w = 0; w < U; ++w)
#pragma unroll
          for (int q = 0; q < B; ++q) y = fmaf(m[w][q], xv[w][q], y);
      }
      part[t] = y;
    }
    __syncthreads();
    const int64_t o = i * B + t;
    float yr = 0.f, rn = 0.f;
    if (t < B) {
#pragma unroll 4
      for (int s = 0; s < PB; ++s) yr += part[t + s * B];
      if constexpr (MODE == kOpS1 || MODE == kOpS3) rn = a.f[o] - yr;
      else if constexpr (MODE == kOpS4 || MODE == kOpS4Dot) rn = a.r[o] - yr;
      rs[t] = rn;
    }
    __syncthreads();
    if (t < B) {
      float tv = 0.f;
      if constexpr (MODE == kOpS1 || MODE == kOpS3 || MODE == kOpS4 || MODE == kOpS4Dot) {
        const float* m = a.dinv + o * B;
#pragma unroll
        for (int q = 0; q < B; ++q) tv = fmaf(m[q], rs[q], tv);
      }
      if constexpr (MODE == kOpS1) {
        const float dn = a.c1 * a.d[o] + a.c2 * tv;
        a.r[o] = rn;
        a.db[o] = dn;
        a.x[o] += dn;
      } else if constexpr (MODE == kOpS2) {
        a.r[o] -= yr;
      } else if constexpr (MODE == kOpS3) {
        const float dn = a.theta_inv * tv;
        a.r[o] = rn;
        a.d[o] = dn;
        a.xb[o] = a.x[o] + dn;
      } else if constexpr (MODE == kOpS4 || MODE == kOpS4Dot) {
        const float z = a.xb[o] + (a.c1 * a.d[o] + a.c2 * tv);
        a.xb[o] = z;
        if constexpr (MODE == kOpS4Dot) dot += (double)a.f[o] * (double)z;
      } else {
        a.q[o] = yr;
        dot += (double)a.p[o] * (double)yr;
      }
    }
    __syncthreads();
  }
  if constexpr (op_has_dot<MODE>()) {
    const double bsum = block_sum(dot, red);
    if (threadIdx.x == 0) a.partial[blockIdx.x] = bsum;
    if (arrive_last(&a.ctrl->counter)) {
      const double tot = sum_partials(a.partial, gridDim.x, 1, 0, red);
      if (threadIdx.x == 0) {
        a.ctrl->counter = 0;
        op_finish<MODE>(a, tot);
      }
    }
  }
}

// Restriction f_c = P^T r of coarse row I by the threads of one CTA (P^T
// values in transposed order, pt_val, so consecutive threads read
// consecutive blocks), fixed-order reduction, then the first Chebyshev step
// of the coarse level: d = D^-1 f / theta, x = d.
template <int BF, int K, int NT>
__device__ __forceinline__ void restrict_row(int64_t I, const int64_t* __restrict__ pt_ptr,
                                             const int32_t* __restrict__ pt_row, const __half* __restrict__ pt_val,
                                             const float* __restrict__ rf, float (&red)[NT / 32][K], float* fout) {
  const int lane = threadIdx.x & 31, w = (threadIdx.x >> 5) % (NT / 32);
  const int tid = threadIdx.x % NT;
  float acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.f;
  for (int64_t e = pt_ptr[I] + tid; e < pt_ptr[I + 1]; e += NT) {
    const int64_t i = pt_row[e];
    float pv[BF * K];
    load_half<BF * K>(pt_val + e * BF * K, pv);
#pragma unroll
    for (int q = 0; q < BF; ++q) {
      const float rv = rf[i * BF + q];
#pragma unroll
      for (int k = 0; k < K; ++k) acc[k] = fmaf(pv[q * K + k], rv, acc[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = warp_sum(acc[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) red[w][k] = acc[k];
  __syncthreads();
  if (tid < K) {
    float s = 0.f;
#pragma unroll
    for (int u = 0; u < NT / 32; ++u) s += red[u][tid];
    fout[tid] = s;
  }
  __syncthreads();
}

template <int BF, int K>
__global__ void __launch_bounds__(128) k_restrict(int64_t n_c, const int64_t* __restrict__ pt_ptr,
                                                  const int32_t* __restrict__ pt_row, const __half* __restrict__ pt_val,
                                                  const float* __restrict__ rf, OpArgs c, const AmgCtrl* ctrl) {
  __shared__ float red[4][K];
  __shared__ float fs[K];
  if (amg_idle(ctrl)) return;
  for (int64_t I = blockIdx.x; I < n_c; I += gridDim.x) {
    restrict_row<BF, K, 128>(I, pt_ptr, pt_row, pt_val, rf, red, fs);
    if (threadIdx.x < K) {
      const int k = threadIdx.x;
      const float* m = c.dinv + (I * K + k) * K;
      float t = 0.f;
#pragma unroll
      for (int q = 0; q < K; ++q) t = fmaf(m[q], fs[q], t);
      const float dn = c.theta_inv * t;
      c.f[I * K + k] = fs[k];
      c.d[I * K + k] = dn;
      c.x[I * K + k] = dn;
    }
  }
}

// Prolongation x += P x_c, one thread per (fine row, component): the
// threads of a row read adjacent rows of its blocks (the FP16 copy of P).
template <int BF, int K>
__global__ void __launch_bounds__(256) k_prolong(int64_t n, const int64_t* __restrict__ p_ptr,
                                                 const int32_t* __restrict__ p_col, const __half* __restrict__ p_val,
                                                 const float* __restrict__ xc, float* __restrict__ x,
                                                 const AmgCtrl* ctrl) {
  if (amg_idle(ctrl)) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * BF) return;
  const int64_t i = t / BF;
  const int r = (int)(t - i * BF);
  float s = 0.f;
  for (int64_t e = p_ptr[i]; e < p_ptr[i + 1]; ++e) {
    float pv[K];
    load_half<K>(p_val + e * BF * K + r * K, pv);  // 4-byte aligned when K is even
    const float* cv = xc + (int64_t)p_col[e] * K;
#pragma unroll
    for (int k = 0; k < K; ++k) s = fmaf(pv[k], cv[k], s);
  }
  x[t] += s;
}

// FP16 copies of P for the V-cycle's transfers: p_h in P order (the
// prolongation) and pt_h in transposed order (block e of P^T is block
// pt_pos[e] of P, the restriction).  Both transfers use the same rounded P,
// so the V-cycle stays symmetric; the Galerkin product uses the FP32 P.
__global__ void k_transfer_copies(int64_t n_e, int bk, const int64_t* __restrict__ pt_pos,
                                  const float* __restrict__ p_val, __half* __restrict__ p_h,
                                  __half* __restrict__ pt_h) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_e * bk) return;
  const int64_t e = t / bk;
  const int c = (int)(t - e * bk);
  const int64_t pos = pt_pos[e];
  pt_h[t] = __float2half_rn(pos >= 0 ? p_val[pos * bk + c] : 0.f);
  p_h[t] = __float2half_rn(p_val[t]);
}

// Restriction onto the coarsest level and its dense solve, one CTA: warps
// over the coarse rows (P^T in transposed order), then x_c = A_c^-1 f_c.
template <int BF, int K>
__global__ void __launch_bounds__(1024) k_coarse_solve(int64_t n_c, const int64_t* __restrict__ pt_ptr,
                                                       const int32_t* __restrict__ pt_row,
                                                       const __half* __restrict__ pt_val, const float* __restrict__ rf,
                                                       const float* __restrict__ inv, float* __restrict__ xc,
                                                       const AmgCtrl* ctrl) {
  __shared__ float fs[kCoarseMaxDof];
  if (amg_idle(ctrl)) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t I = w; I < n_c; I += blockDim.x >> 5) {
    float acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.f;
    for (int64_t e = pt_ptr[I] + lane; e < pt_ptr[I + 1]; e += 32) {
      const int64_t i = pt_row[e];
      float pv[BF * K];
      load_half<BF * K>(pt_val + e * BF * K, pv);
#pragma unroll
      for (int q = 0; q < BF; ++q) {
        const float rv = rf[i * BF + q];
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = fmaf(pv[q * K + k], rv, acc[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = warp_sum(acc[k]);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < K; ++k) fs[I * K + k] = acc[k];
  }
  __syncthreads();
  const int m = (int)(n_c * K);
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < m; ++j) s = fmaf(inv[(int64_t)t * m + j], fs[j], s);
    xc[t] = s;
  }
}

// ------------------------------------------------------- fused coarse cycle --
// Everything of a V-cycle below level 0 -- restriction from level 0, the
// Chebyshev passes of every coarser level, the coarsest solve and the
// prolongations back to level 0 -- as one cooperative launch: phases
// separated by grid barriers, instead of about fourteen short launches whose
// work (a few thousand rows, or 96) is mostly launch and tail latency.
//
// Work decomposition: a warp per block row of a coarse operator (lanes hold
// (block, row) items, 32 / K blocks per pass, partial rows summed across
// lanes by shuffles in a fixed order), a warp per coarse row of a
// restriction, a thread per (fine row, component) of a prolongation, and CTA
// 0 for the coarsest solve; a level with no more rows than the grid has CTAs
// takes a CTA per row instead of a warp.  Every sum keeps a fixed order, so results are
// identical run to run; the arithmetic is that of the per-level kernels
// above up to the order of partial row sums.
#ifndef TFG_CYC_THREADS
#define TFG_CYC_THREADS 512
#endif
#ifndef TFG_CYC_PER_SM
#define TFG_CYC_PER_SM 2
#endif
constexpr int kCycT = TFG_CYC_THREADS;    // threads per CTA
constexpr int kCycPerSm = TFG_CYC_PER_SM;  // CTAs per SM at most (occupancy may allow fewer)
constexpr long long kCycSpin = 4000000000LL;  // clock cycles a barrier wait may last (about 2 s)

struct CycLevel {
  int64_t n;  // block rows
  const int64_t* a_ptr;
  const int32_t* a_col;
  const float* a_val;
  const float* dinv;
  float *f, *x, *xb, *r, *d, *db;
  float theta_inv, c1, c2;
  // transfer to the next level
  const int64_t* p_ptr;
  const int32_t* p_col;
  const __half* p_h;
  const int64_t* pt_ptr;
  const int32_t* pt_row;
  const __half* pt_val;
};

// Arrival counter and error flag of the fused cycle's grid barriers (one
// per handle, zeroed at the start of every solve).
struct CycBarrier {
  unsigned long long seq;
  int error;
};

struct CycArgs {
  int n_levels;
  CycLevel L[kMaxLevels];
  const float* coarse_inv;
  AmgCtrl* ctrl;
  CycBarrier* bar;
};

// Grid barrier with a bounded wait: one monotonic 64-bit arrival counter per
// solve, release add by thread 0 of each CTA after a CTA barrier (cumulative:
// it publishes the CTA's writes), relaxed polling with a short sleep, one
// acquire fence.  A wait that runs out sets the error flag and the CG's
// done code; returns false on every thread once any CTA's wait ran out.
// Grid barrier of the fused cycle.  The counter only grows (it is zeroed
// once per solve), so every barrier of a launch has a known target: the
// first one learns the launch's base from the value its atomic returns, the
// later ones arrive with a fire-and-forget release reduction (no round trip)
// and poll for base + (j + 1) x grid.  `next` (thread 0's copy) carries the
// target of the next barrier.  The wait is bounded (kCycSpin cycles); a
// timeout flags the barrier and the solve.
__device__ __forceinline__ bool cyc_barrier(CycBarrier* b, AmgCtrl* c, unsigned long long& next) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long target;
    if (next == 0ull) {
      unsigned long long old;
      asm volatile("atom.add.release.gpu.u64 %0, [%1], 1;" : "=l"(old) : "l"(&b->seq) : "memory");
      target = (old / gridDim.x + 1) * gridDim.x;
    } else {
      asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(&b->seq) : "memory");
      target = next;
    }
    next = target + gridDim.x;
    const long long t0 = clock64();
    int good = 1;
    while (true) {
      unsigned long long now;
      asm volatile("ld.relaxed.gpu.u64 %0, [%1];" : "=l"(now) : "l"(&b->seq) : "memory");
      if (now >= target) break;
      if (*(volatile int*)&b->error) {
        good = 0;
        break;
      }
      if (clock64() - t0 > kCycSpin) {
        atomicExch(&b->error, 1);
        atomicExch(&c->done, kBarrierTimeout);
        good = 0;
        break;
      }
      __nanosleep(32);
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// One Chebyshev pass of a coarse level on block row i by one warp (the
// modes S1..S4 of op_epilogue).
template <int K, int MODE>
__device__ __forceinline__ void cyc_row(const CycLevel& L, int64_t i, int lane, uint64_t pol) {
  constexpr int PB = 32 / K;  // blocks per pass
  constexpr int U = 2;        // passes with loads in flight together
  const float* __restrict__ v = MODE == kOpS1 || MODE == kOpS4 ? L.d : MODE == kOpS2 ? L.db : L.x;
  const int blk = lane / K, r = lane - (lane / K) * K;
  float y = 0.f;
  if (blk < PB) {
    const int64_t e1 = L.a_ptr[i + 1];
    for (int64_t e = L.a_ptr[i] + blk; e < e1; e += U * PB) {
      int64_t c[U];
#pragma unroll
      for (int w = 0; w < U; ++w) c[w] = e + w * PB < e1 ? (int64_t)ld_l2(L.a_col + e + w * PB, pol) : -1;
      float m[U][K], xv[U][K];
#pragma unroll
      for (int w = 0; w < U; ++w)
#pragma unroll
        for (int q = 0; q < K; ++q) {
          m[w][q] = c[w] >= 0 ? ld_l2(L.a_val + (e + w * PB) * K * K + r * K + q, pol) : 0.f;
          xv[w][q] = c[w] >= 0 ? v[c[w] * K + q] : 0.f;
        }
#pragma unroll
      for (int w = 0; w < U; ++w)
#pragma unroll
        for (int q = 0; q < K; ++q) y = fmaf(m[w][q], xv[w][q], y);
    }
  }
  // lane r (< K) adds the lanes r + b K, b = 1 .. PB-1, in order
  float t = y;
#pragma unroll
  for (int b = 1; b < PB; ++b) t += __shfl_sync(0xffffffffu, y, (r + b * K) & 31);
  const int64_t o = i * K + r;
  float rn = 0.f;
  if (lane < K) {
    if constexpr (MODE == kOpS1 || MODE == kOpS3) rn = L.f[o] - t;
    else if constexpr (MODE == kOpS4) rn = L.r[o] - t;
  }
  float tv = 0.f;
  if constexpr (MODE != kOpS2) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const float rq = __shfl_sync(0xffffffffu, rn, q);
      if (lane < K) tv = fmaf(L.dinv[o * K + q], rq, tv);
    }
  }
  if (lane < K) {
    if constexpr (MODE == kOpS1) {
      const float dn = L.c1 * L.d[o] + L.c2 * tv;
      L.r[o] = rn;
      L.db[o] = dn;
      L.x[o] += dn;
    } else if constexpr (MODE == kOpS2) {
      L.r[o] -= t;
    } else if constexpr (MODE == kOpS3) {
      const float dn = L.theta_inv * tv;
      L.r[o] = rn;
      L.d[o] = dn;
      L.xb[o] = L.x[o] + dn;
    } else {
      L.xb[o] = L.xb[o] + (L.c1 * L.d[o] + L.c2 * tv);
    }
  }
}

// Restriction f_c = P^T r of coarse row I by one warp (P^T in transposed
// order, FP16), xor-tree sums, then the first Chebyshev step of the coarse
// level: d = D^-1 f / theta, x = d.
template <int BF, int K>
__device__ __forceinline__ void cyc_restrict(const CycLevel& F, const CycLevel& C, int64_t I, int lane) {
  float acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.f;
  for (int64_t e = F.pt_ptr[I] + lane; e < F.pt_ptr[I + 1]; e += 32) {
    const int64_t i = F.pt_row[e];
    float pv[BF * K];
    load_half<BF * K>(F.pt_val + e * BF * K, pv);
#pragma unroll
    for (int q = 0; q < BF; ++q) {
      const float rv = F.r[i * BF + q];
#pragma unroll
      for (int k = 0; k < K; ++k) acc[k] = fmaf(pv[q * K + k], rv, acc[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = warp_sum(acc[k]);
  if (lane < K) {
    float t = 0.f, fk = 0.f;
#pragma unroll
    for (int q = 0; q < K; ++q) {
      t = fmaf(C.dinv[(I * K + lane) * K + q], acc[q], t);
      if (q == lane) fk = acc[q];
    }
    const float dn = C.theta_inv * t;
    C.f[I * K + lane] = fk;
    C.d[I * K + lane] = dn;
    C.x[I * K + lane] = dn;
  }
}

// Restriction onto the coarsest level and its dense solve, by one CTA.
template <int BF, int K>
__device__ __forceinline__ void cyc_coarsest(const CycLevel& F, const CycLevel& C, const float* __restrict__ inv,
                                             float* fs) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t I = w; I < C.n; I += kCycT / 32) {
    float acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.f;
    for (int64_t e = F.pt_ptr[I] + lane; e < F.pt_ptr[I + 1]; e += 32) {
      const int64_t i = F.pt_row[e];
      float pv[BF * K];
      load_half<BF * K>(F.pt_val + e * BF * K, pv);
#pragma unroll
      for (int q = 0; q < BF; ++q) {
        const float rv = F.r[i * BF + q];
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = fmaf(pv[q * K + k], rv, acc[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = warp_sum(acc[k]);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < K; ++k) fs[I * K + k] = acc[k];
  }
  __syncthreads();
  const int m = (int)(C.n * K);
  for (int t = threadIdx.x; t < m; t += kCycT) {
    float s = 0.f;
    for (int j = 0; j < m; ++j) s = fmaf(inv[(int64_t)t * m + j], fs[j], s);
    C.xb[t] = s;
  }
}

// Prolongation x += P x_c, a thread per (fine row, component), threads
// t0, t0 + stride, ...; each thread keeps kProlongU items' loads in flight
// (every item still sums its blocks in ascending order).
constexpr int kProlongU = 4;
template <int BF, int K>
__device__ __forceinline__ void cyc_prolong(const CycLevel& F, const float* __restrict__ xc, float* __restrict__ x,
                                            int64_t t0, int64_t stride) {
  const int64_t n = F.n * BF;
  for (int64_t t = t0; t < n; t += kProlongU * stride) {
    int64_t e[kProlongU], e1[kProlongU];
    float s[kProlongU];
#pragma unroll
    for (int u = 0; u < kProlongU; ++u) {
      const int64_t tu = t + u * stride;
      s[u] = 0.f;
      e[u] = e1[u] = 0;
      if (tu < n) {
        const int64_t i = tu / BF;
        e[u] = F.p_ptr[i];
        e1[u] = F.p_ptr[i + 1];
      }
    }
    bool more = true;
    while (more) {
      more = false;
#pragma unroll
      for (int u = 0; u < kProlongU; ++u) {
        if (e[u] < e1[u]) {
          const int64_t tu = t + u * stride;
          const int r = (int)(tu - (tu / BF) * BF);
          float pv[K];
          load_half<K>(F.p_h + e[u] * BF * K + r * K, pv);
          const float* cv = xc + (int64_t)F.p_col[e[u]] * K;
#pragma unroll
          for (int k = 0; k < K; ++k) s[u] = fmaf(pv[k], cv[k], s[u]);
          ++e[u];
          more = true;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kProlongU; ++u) {
      const int64_t tu = t + u * stride;
      if (tu < n) x[tu] += s[u];
    }
  }
}

template <int K, int MODE>
__device__ __forceinline__ void cyc_pass(const CycLevel& L, int lane, int64_t warp, int64_t n_warps, uint64_t pol) {
  for (int64_t i = warp; i < L.n; i += n_warps) cyc_row<K, MODE>(L, i, lane, pol);
}

// The same pass on block row i by a whole CTA, for levels with fewer rows
// than the grid has CTAs (their rows are long: the operator fills in as the
// levels coarsen).  Thread t < PB K holds (block t / K, row t % K) items;
// the PB partial rows are summed in shared memory in a fixed order.
template <int K, int MODE>
__device__ __forceinline__ void cyc_row_cta(const CycLevel& L, int64_t i, uint64_t pol, float* part) {
  constexpr int PB = kCycT / K;
  const int t = threadIdx.x;
  const float* __restrict__ v = MODE == kOpS1 || MODE == kOpS4 ? L.d : MODE == kOpS2 ? L.db : L.x;
  const int blk = t / K, r = t - (t / K) * K;
  float y = 0.f;
  if (blk < PB) {
    const int64_t e1 = L.a_ptr[i + 1];
    for (int64_t e = L.a_ptr[i] + blk; e < e1; e += PB) {
      const int64_t c = ld_l2(L.a_col + e, pol);
#pragma unroll
      for (int q = 0; q < K; ++q) y = fmaf(ld_l2(L.a_val + e * K * K + r * K + q, pol), v[c * K + q], y);
    }
  }
  part[t] = y;
  __syncthreads();
  __shared__ float rs[8];
  const int64_t o = i * K + t;
  float yr = 0.f, rn = 0.f;
  if (t < K) {
    for (int b = 0; b < PB; ++b) yr += part[t + b * K];
    if constexpr (MODE == kOpS1 || MODE == kOpS3) rn = L.f[o] - yr;
    else if constexpr (MODE == kOpS4) rn = L.r[o] - yr;
    rs[t] = rn;
  }
  __syncthreads();
  if (t < K) {
    float tv = 0.f;
    if constexpr (MODE != kOpS2) {
#pragma unroll
      for (int q = 0; q < K; ++q) tv = fmaf(L.dinv[o * K + q], rs[q], tv);
    }
    if constexpr (MODE == kOpS1) {
      const float dn = L.c1 * L.d[o] + L.c2 * tv;
      L.r[o] = rn;
      L.db[o] = dn;
      L.x[o] += dn;
    } else if constexpr (MODE == kOpS2) {
      L.r[o] -= yr;
    } else if constexpr (MODE == kOpS3) {
      const float dn = L.theta_inv * tv;
      L.r[o] = rn;
      L.d[o] = dn;
      L.xb[o] = L.x[o] + dn;
    } else {
      L.xb[o] = L.xb[o] + (L.c1 * L.d[o] + L.c2 * tv);
    }
  }
  __syncthreads();
}

// Restriction onto coarse row I by a whole CTA (coarse levels with no more
// rows than the grid has CTAs): threads over the row's P^T entries, warp
// xor-trees, then the warps' sums in order; then the first Chebyshev step.
template <int BF, int K>
__device__ __forceinline__ void cyc_restrict_cta(const CycLevel& F, const CycLevel& C, int64_t I, float* part) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  constexpr int NWp = kCycT / 32;
  float acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.f;
  for (int64_t e = F.pt_ptr[I] + t; e < F.pt_ptr[I + 1]; e += kCycT) {
    const int64_t i = F.pt_row[e];
    float pv[BF * K];
    load_half<BF * K>(F.pt_val + e * BF * K, pv);
#pragma unroll
    for (int q = 0; q < BF; ++q) {
      const float rv = F.r[i * BF + q];
#pragma unroll
      for (int k = 0; k < K; ++k) acc[k] = fmaf(pv[q * K + k], rv, acc[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = warp_sum(acc[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) part[w * K + k] = acc[k];
  __syncthreads();
  __shared__ float fsum[8];
  if (t < K) {
    float f = 0.f;
    for (int u = 0; u < NWp; ++u) f += part[u * K + t];
    fsum[t] = f;
  }
  __syncthreads();
  if (t < K) {
    float tv = 0.f;
#pragma unroll
    for (int q = 0; q < K; ++q) tv = fmaf(C.dinv[(I * K + t) * K + q], fsum[q], tv);
    const float dn = C.theta_inv * tv;
    C.f[I * K + t] = fsum[t];
    C.d[I * K + t] = dn;
    C.x[I * K + t] = dn;
  }
  __syncthreads();
}

// One pass over a coarse level: a warp per row, or a CTA per row when the
// level has no more rows than the grid has CTAs.
template <int K, int MODE>
__device__ __forceinline__ void cyc_level_pass(const CycLevel& L, int lane, int64_t warp, int64_t n_warps,
                                               uint64_t pol, float* part) {
  if (L.n <= (int64_t)gridDim.x) {
    for (int64_t i = blockIdx.x; i < L.n; i += gridDim.x) cyc_row_cta<K, MODE>(L, i, pol, part);
  } else {
    cyc_pass<K, MODE>(L, lane, warp, n_warps, pol);
  }
}

template <int B0, int K>
__global__ void __launch_bounds__(kCycT) k_coarse_cycle(CycArgs a) {
  __shared__ float fs[kCoarseMaxDof];
  __shared__ float part[kCycT];
  AmgCtrl* c = a.ctrl;
  CycBarrier* bar = a.bar;
  if (amg_idle(c)) return;
  unsigned long long next = 0;  // target of the next grid barrier (thread 0)
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * kCycT + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * kCycT) >> 5;
  const int64_t tid = (int64_t)blockIdx.x * kCycT + threadIdx.x;
  const int64_t n_threads = (int64_t)gridDim.x * kCycT;
  const uint64_t pol = l2_policy(true);
  const int last = a.n_levels - 1;
  // down: restrict (with the first Chebyshev step), then the level's second
  // pass and residual
  for (int l = 0; l < last; ++l) {
    const CycLevel& F = a.L[l];
    const CycLevel& C = a.L[l + 1];
    if (l + 1 == last) {
      if (blockIdx.x == 0) {
        if (l == 0) cyc_coarsest<B0, K>(F, C, a.coarse_inv, fs);
        else cyc_coarsest<K, K>(F, C, a.coarse_inv, fs);
      }
      break;
    }
    if (C.n <= (int64_t)gridDim.x) {
      for (int64_t I = blockIdx.x; I < C.n; I += gridDim.x) {
        if (l == 0) cyc_restrict_cta<B0, K>(F, C, I, part);
        else cyc_restrict_cta<K, K>(F, C, I, part);
      }
    } else {
      for (int64_t I = warp; I < C.n; I += n_warps) {
        if (l == 0) cyc_restrict<B0, K>(F, C, I, lane);
        else cyc_restrict<K, K>(F, C, I, lane);
      }
    }
    if (!cyc_barrier(bar, c, next)) return;
    cyc_level_pass<K, kOpS1>(C, lane, warp, n_warps, pol, part);
    if (!cyc_barrier(bar, c, next)) return;
    cyc_level_pass<K, kOpS2>(C, lane, warp, n_warps, pol, part);
    if (!cyc_barrier(bar, c, next)) return;
  }
  // up: prolongate, then the level's post-smoothing; level 0 continues in
  // the next launch
  for (int l = last - 1; l >= 0; --l) {
    if (!cyc_barrier(bar, c, next)) return;
    const CycLevel& F = a.L[l];
    if (l == 0) {
      cyc_prolong<B0, K>(F, a.L[1].xb, F.x, tid, n_threads);
      break;
    }
    cyc_prolong<K, K>(F, a.L[l + 1].xb, F.x, tid, n_threads);
    if (!cyc_barrier(bar, c, next)) return;
    cyc_level_pass<K, kOpS3>(F, lane, warp, n_warps, pol, part);
    if (!cyc_barrier(bar, c, next)) return;
    cyc_level_pass<K, kOpS4>(F, lane, warp, n_warps, pol, part);
  }
}

// ---------------------------------------------------------------- CG ------
// p = z + beta p.
__global__ void __launch_bounds__(256) k_pup(int64_t n, const float* __restrict__ z, float* __restrict__ p,
                                             const AmgCtrl* ctrl) {
  if (amg_idle(ctrl)) return;
  const float beta = (float)ctrl->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// ||b||^2, the first residual scale and the tolerances.
__global__ void __launch_bounds__(256) k_cg_bnorm(int64_t n, const double* __restrict__ b, double rtol2,
                                                  double* __restrict__ partial, AmgCtrl* ctrl) {
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
      const double sc = unit_scale(bb);
      ctrl->bb = bb;
      ctrl->rscale = sc;
      ctrl->tol2bb = rtol2 * bb;
      ctrl->tol2_lo = rtol2 * bb * sc * sc;
    }
  }
}

// Level-0 first Chebyshev step on a fresh residual: d = D^-1 r / theta, x = d.
template <int D>
__device__ __forceinline__ void pre_step(const float* __restrict__ dinv, float theta_inv, int64_t i,
                                         const float (&rv)[D], float* __restrict__ d, float* __restrict__ x) {
  float t[D];
  block_mv<D>(dinv + i * D * D, rv, t);
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const float dn = theta_inv * t[c];
    d[i * D + c] = dn;
    x[i * D + c] = dn;
  }
}

// x = 0: r = b * rscale, ||r||^2, first smoothing step.
template <int D>
__global__ void __launch_bounds__(256) k_cg_init(int64_t n_nod, const double* __restrict__ b, float* __restrict__ r,
                                                 const float* __restrict__ dinv, float theta_inv, float* __restrict__ d,
                                                 float* __restrict__ mx, double* __restrict__ partial, AmgCtrl* ctrl) {
  __shared__ double red[32];
  const double sc = ctrl->rscale;
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nod; i += (int64_t)gridDim.x * blockDim.x) {
    float rv[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      rv[c] = (float)(b[i * D + c] * sc);
      r[i * D + c] = rv[c];
      rr += (double)rv[c] * (double)rv[c];
    }
    pre_step<D>(dinv, theta_inv, i, rv, d, mx);
  }
  rr = block_sum(rr, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = rr;
  if (arrive_last(&ctrl->counter)) {
    const double t = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      ctrl->rr = t;
      ctrl->rr_ref = t;
      ctrl->rr_true = ctrl->bb;
      ctrl->rz = 1.0;
      ctrl->pscale = 0.0;
      ctrl->iters = 0;
      ctrl->replacements = 0;
      ctrl->replace = 0;
      if (!isfinite(t) || !isfinite(ctrl->bb)) ctrl->done = kNonFinite;
      else if (ctrl->bb == 0.0 || t <= ctrl->tol2_lo) ctrl->done = kConverged;
      else ctrl->done = kRun;
    }
  }
}

// x_lo += alpha p; r -= alpha q; ||r||^2; first smoothing step of the next
// cycle; convergence or replacement decision.
template <int D>
__global__ void __launch_bounds__(256) k_cg_update(int64_t n_nod, float* __restrict__ xlo, float* __restrict__ r,
                                                   const float* __restrict__ p, const float* __restrict__ q,
                                                   const float* __restrict__ dinv, float theta_inv,
                                                   float* __restrict__ d, float* __restrict__ mx,
                                                   double* __restrict__ partial, AmgCtrl* ctrl) {
  __shared__ double red[32];
  pdl_enter();
  if (amg_idle(ctrl)) return;
  const float alpha = (float)ctrl->alpha;
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nod; i += (int64_t)gridDim.x * blockDim.x) {
    float rv[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const int64_t k = i * D + c;
      xlo[k] += alpha * p[k];
      rv[c] = r[k] - alpha * q[k];
      r[k] = rv[c];
      rr += (double)rv[c] * (double)rv[c];
    }
    pre_step<D>(dinv, theta_inv, i, rv, d, mx);
  }
  rr = block_sum(rr, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = rr;
  if (arrive_last(&ctrl->counter)) {
    const double t = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      AmgCtrl* c = ctrl;
      c->counter = 0;
      c->iters += 1;
      c->rr = t;
      if (!isfinite(t)) {
        c->done = kNonFinite;
      } else if (c->mixed) {
        if (t <= c->tol2_lo || t <= c->delta2 * c->rr_ref) c->replace = 1;
      } else if (t <= c->tol2_lo) {
        c->done = kConverged;
      }
      if (c->done == kRun && !c->replace && c->iters >= c->max_iter) c->done = kMaxIter;
    }
  }
}

// x64 += x_lo / rscale; x_lo = 0.
__global__ void k_cg_fold(int64_t n, double* __restrict__ x64, float* __restrict__ xlo, const AmgCtrl* ctrl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x64[i] += (double)xlo[i] * (1.0 / ctrl->rscale);
  xlo[i] = 0.f;
}

// FP64 replacement: r = (b - y) * s with s the unit scale of the current
// residual estimate, first smoothing step, FP64 convergence decision.  CG
// restarts (pscale = 0: p = z): each inner run reduces the residual by delta
// (1e-4 and below), deep enough that the gap FP32 rounding leaves between the
// recursive and the true residual is a sizeable part of the new residual, and
// a direction kept across it loses conjugacy (measured: 55 iterations for one
// 1e-4 reduction instead of 8).  Each restart is iterative refinement with an
// inner multigrid CG.
template <int D>
__global__ void __launch_bounds__(256) k_cg_replace(int64_t n_nod, const double* __restrict__ b,
                                                    const double* __restrict__ y, float* __restrict__ r,
                                                    const float* __restrict__ dinv, float theta_inv,
                                                    float* __restrict__ d, float* __restrict__ mx,
                                                    double* __restrict__ partial, AmgCtrl* ctrl) {
  __shared__ double red[32];
  const double sc_old = ctrl->rscale;
  const double sc = unit_scale(ctrl->rr / (sc_old * sc_old));
  double rr = 0.0, r64 = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nod; i += (int64_t)gridDim.x * blockDim.x) {
    float rv[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const int64_t k = i * D + c;
      const double rd = b[k] - y[k];
      r64 += rd * rd;
      rv[c] = (float)(rd * sc);
      r[k] = rv[c];
      rr += (double)rv[c] * (double)rv[c];
    }
    pre_step<D>(dinv, theta_inv, i, rv, d, mx);
  }
  const double s1 = block_sum(rr, red);
  const double s2 = block_sum(r64, red);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s1;
    partial[2 * blockIdx.x + 1] = s2;
  }
  if (arrive_last(&ctrl->counter)) {
    const double t1 = sum_partials(partial, gridDim.x, 2, 0, red);
    const double t2 = sum_partials(partial, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      AmgCtrl* c = ctrl;
      c->counter = 0;
      c->rr_true = t2;
      c->replacements += 1;
      c->replace = 0;
      if (!isfinite(t1) || !isfinite(t2)) {
        c->done = kNonFinite;
      } else if (t2 <= c->tol2bb) {
        c->done = kConverged;
      } else if (c->done == kRun) {
        c->rr = t1;
        c->rr_ref = t1;
        c->pscale = 0.0;
        c->rscale = sc;
        c->tol2_lo = c->tol2bb * sc * sc;
      }
    }
  }
}

// FP32-only solve: x64 = x_lo / rscale.
__global__ void k_cg_out(int64_t n, const float* __restrict__ xlo, double* __restrict__ x64, const AmgCtrl* ctrl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x64[i] = (double)xlo[i] * (1.0 / ctrl->rscale);
}

// ------------------------------------------------------- CG-Lanczos -----
// Jacobi-preconditioned CG on a fixed pseudo-random right-hand side; its
// coefficients give the Lanczos tridiagonal of D^-1 A.
template <int B>
__global__ void __launch_bounds__(256) k_lz_init(int64_t n, const float* __restrict__ dinv, float* __restrict__ r,
                                                 float* __restrict__ z, float* __restrict__ p,
                                                 double* __restrict__ partial, AmgCtrl* ctrl) {
  __shared__ double red[32];
  double rz = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float rv[B], zv[B];
#pragma unroll
    for (int c = 0; c < B; ++c) {
      const uint32_t h = amg_hash((uint32_t)(i * B + c) ^ 0x9e3779b9U);
      rv[c] = (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;
      r[i * B + c] = rv[c];
    }
    block_mv<B>(dinv + i * B * B, rv, zv);
#pragma unroll
    for (int c = 0; c < B; ++c) {
      z[i * B + c] = zv[c];
      p[i * B + c] = zv[c];
      rz += (double)rv[c] * (double)zv[c];
    }
  }
  rz = block_sum(rz, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = rz;
  if (arrive_last(&ctrl->counter)) {
    const double t = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      ctrl->rz = t;
      ctrl->lz_step = 0;
      ctrl->replace = 0;
      ctrl->done = (isfinite(t) && t > 0.0) ? kRun : kBreakdown;
    }
  }
}

template <int B>
__global__ void __launch_bounds__(256) k_lz_update(int64_t n, const float* __restrict__ dinv, float* __restrict__ r,
                                                   float* __restrict__ z, const float* __restrict__ q,
                                                   double* __restrict__ partial, AmgCtrl* ctrl,
                                                   double* __restrict__ lz) {
  __shared__ double red[32];
  if (amg_idle(ctrl)) return;
  const float alpha = (float)ctrl->alpha;
  double rz = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float rv[B], zv[B];
#pragma unroll
    for (int c = 0; c < B; ++c) {
      rv[c] = r[i * B + c] - alpha * q[i * B + c];
      r[i * B + c] = rv[c];
    }
    block_mv<B>(dinv + i * B * B, rv, zv);
#pragma unroll
    for (int c = 0; c < B; ++c) {
      z[i * B + c] = zv[c];
      rz += (double)rv[c] * (double)zv[c];
    }
  }
  rz = block_sum(rz, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = rz;
  if (arrive_last(&ctrl->counter)) {
    const double t = sum_partials(partial, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      ctrl->counter = 0;
      if (!(isfinite(t) && t > 0.0)) {
        ctrl->done = kBreakdown;
      } else {
        ctrl->beta = t / ctrl->rz;
        lz[2 * ctrl->lz_step + 1] = ctrl->beta;
        ctrl->rz = t;
        ctrl->lz_step += 1;
      }
    }
  }
}

// Largest eigenvalue of the symmetric tridiagonal (diag a, off-diagonal b) by
// Sturm-sequence bisection.
double tridiag_max_eig(const std::vector<double>& a, const std::vector<double>& b) {
  const int k = (int)a.size();
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < k; ++i) {
    const double rad = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < k ? fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - rad);
    hi = std::max(hi, a[i] + rad);
  }
  auto count_below = [&](double x) {  // eigenvalues < x
    int cnt = 0;
    double q = 1.0;
    for (int i = 0; i < k; ++i) {
      const double off = i > 0 ? b[i - 1] * b[i - 1] : 0.0;
      q = a[i] - x - (i > 0 ? off / q : 0.0);
      if (q == 0.0) q = -1e-300;
      if (q < 0.0) ++cnt;
    }
    return cnt;
  };
  for (int it = 0; it < 200 && hi - lo > 1e-12 * std::max(1.0, fabs(hi)); ++it) {
    const double mid = 0.5 * (lo + hi);
    if (count_below(mid) >= k) hi = mid;
    else lo = mid;
  }
  return hi;
}

}  // namespace

// ================================================================= handle ==
struct AmgLevel {
  int64_t n = 0;  // block rows
  int b = 0;      // block size
  Graph g{};      // aggregation graph (level 0: mesh node graph; coarser: operator pattern)
  // operator of a coarser level (block CSR, owned)
  int64_t* a_ptr = nullptr;
  int32_t* a_col = nullptr;
  float* a_val = nullptr;
  int64_t a_nnz = 0;
  float* dinv = nullptr;
  // transfer to the next level
  int32_t* agg = nullptr;
  int64_t n_agg = 0;
  float* tval = nullptr;
  int64_t* p_ptr = nullptr;
  int32_t* p_col = nullptr;
  float* p_val = nullptr;
  int64_t p_nnz = 0;
  int64_t* pt_ptr = nullptr;
  int32_t* pt_row = nullptr;
  int64_t* pt_pos = nullptr;
  __half* pt_val = nullptr;  // FP16 P values in transposed order (restriction)
  __half* p_h = nullptr;     // FP16 P values in P order (prolongation)
  int64_t* ap_ptr = nullptr;
  int32_t* ap_col = nullptr;
  float* ap_val = nullptr;
  int64_t ap_nnz = 0;
  // contribution lists of the blocks of A P
  int64_t* wl_ptr = nullptr;  // [ap_nnz + 1]
  int32_t* wl_k = nullptr;    // neighbour slot (block of A) of each contribution
  int32_t* wl_p = nullptr;    // P block of each contribution
  int32_t* ap_row = nullptr;  // [ap_nnz] fine row of each block
  // Galerkin contribution lists of the next level's blocks
  int64_t* cl_ptr = nullptr;  // [C.a_nnz + 1]
  int32_t* cl_p = nullptr;    // P block of each contribution
  int32_t* cl_w = nullptr;    // A P block of each contribution
  int32_t* slot_row = nullptr;  // [C.a_nnz] coarse row of each block
  // contribution lists of the blocks of A T (smoothed prolongator)
  int64_t* tl_ptr = nullptr;  // [p_nnz + 1]
  int32_t* tl_k = nullptr;    // neighbour slot of each contribution
  int32_t* p_row = nullptr;   // [p_nnz] fine row of each block
  // smoother
  double rho = 0.0;
  float theta_inv = 0.f, c1 = 0.f, c2 = 0.f;
  // vectors (level 0: f and xb are the CG residual and preconditioned residual)
  float *f = nullptr, *x = nullptr, *xb = nullptr, *r = nullptr, *d = nullptr, *db = nullptr;
};

}  // namespace tfg

struct fem_amg {
  int dim = 0, K = 0, n_levels = 0;
  tfg::AmgLevel L[tfg::kMaxLevels];
  float* coarse_inv = nullptr;
  double* coarse_work = nullptr;
  int64_t m_coarse = 0;
  uint8_t* active = nullptr;  // level 0: nodes with a free DOF
  // CG state
  float *xlo = nullptr, *rcg = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  tfg::AmgCtrl* ctrl = nullptr;
  tfg::AmgCtrl* lzc = nullptr;
  double* lz = nullptr;
  double* partial = nullptr;
  int32_t* status = nullptr;
  unsigned long long* counter = nullptr;
  std::vector<void*> mem;
  int64_t dropped = 0;
  bool ready = false;
  // CUDA events around the level-0 SpMV launches of a chunk (timing on)
  static constexpr int kTimed = 32;
  cudaEvent_t ev[2 * kTimed];
  bool ev_ready = false;
  int ev_used = kTimed;  // events are recorded only inside a timed chunk
  double timed_ms = 0.0;
  long long timed_n = 0;
  // level-0 operator captured at setup
  const int64_t* sell_base = nullptr;
  const int32_t* sell_col = nullptr;
  const float* sell_val = nullptr;
  const float* dinv0 = nullptr;  // the hierarchy's own copy of the setup matrix's block-Jacobi inverse
  float* dinv0_own = nullptr;
  int64_t dinv0_len = 0;
  // FP16 smoothing copy of the level-0 matrix (allocated at the first setup)
  __half* sv16 = nullptr;
  int64_t sv16_len = 0;
  float* s16inv = nullptr;
  unsigned int* absmax = nullptr;
  // fused coarse cycle: CTAs (0 not yet sized, -1 unavailable) and barrier state
  int cyc_blocks = 0;
  tfg::CycBarrier* cyc_bar = nullptr;

  template <typename T>
  T* alloc(int64_t count, cudaStream_t st) {
    void* p = nullptr;
    const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
    (void)st;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    mem.push_back(p);
    return static_cast<T*>(p);
  }
};

namespace tfg {
namespace {

constexpr int kPartialLen = 8192;

int read_u64(const unsigned long long* d, unsigned long long* h, cudaStream_t st) {
  if (cudaMemcpyAsync(h, d, sizeof(*h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("AMG read");
  return FEM_OK;
}

int read_i64(const int64_t* d, int64_t* h, cudaStream_t st) {
  if (cudaMemcpyAsync(h, d, sizeof(*h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("AMG read");
  return FEM_OK;
}

int read_status(fem_amg* h, cudaStream_t st, const char* what) {
  int32_t s = 0;
  if (cudaMemcpyAsync(&s, h->status, sizeof(s), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda(what);
  if (s & kStatBounds) {
    set_last_error("%s: a row of the multigrid hierarchy exceeds its size limit", what);
    return FEM_BOUNDS;
  }
  if (s & kStatNonFinite) {
    set_last_error("%s: singular or non-finite block in the multigrid hierarchy", what);
    return FEM_NONFINITE;
  }
  return FEM_OK;
}

// Exclusive scan of cnt [n] into ptr [n+1]; returns the total on the host.
int scan_total(fem_amg* h, const int64_t* cnt, int64_t* ptr, int64_t n, int64_t* total, cudaStream_t st) {
  int64_t* ws = h->alloc<int64_t>((int64_t)(scan_workspace_bytes(n) / sizeof(int64_t)) + 1, st);
  if (!ws) return check_cuda("AMG scan workspace");
  int rc = scan_exclusive(cnt, ptr, n, ws, st);
  if (rc) return rc;
  return read_i64(ptr + n, total, st);
}

// Aggregation of level l's graph into h->L[l].agg; returns the aggregate count.
int aggregate(fem_amg* h, int l, const uint8_t* con, cudaStream_t st) {
  AmgLevel& L = h->L[l];
  const int64_t n = L.n;
  uint8_t* active = l == 0 ? h->active : h->alloc<uint8_t>(n, st);
  uint8_t* state = h->alloc<uint8_t>(n, st);
  uint64_t* k1 = h->alloc<uint64_t>(n, st);
  int64_t* flags = h->alloc<int64_t>(n, st);
  int64_t* ids = h->alloc<int64_t>(n + 1, st);
  int32_t* agg2 = h->alloc<int32_t>(n, st);
  L.agg = h->alloc<int32_t>(n, st);
  if (!active || !state || !k1 || !flags || !ids || !agg2 || !L.agg) return check_cuda("AMG aggregation buffers");
  const unsigned gn = grid_for(n, kT);
  k_agg_active<<<gn, kT, 0, st>>>(n, L.b, l == 0 ? con : nullptr, active, state);
  note_launch();
  for (int round = 0;; ++round) {
    if (round > 10000) {
      set_last_error("AMG aggregation: the independent-set rounds did not terminate");
      return FEM_CUDA_ERROR;
    }
    cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), st);
    k_mis_max1<<<gn, kT, 0, st>>>(L.g, active, state, k1);
    note_launch();
    k_mis_max2<<<gn, kT, 0, st>>>(L.g, active, state, k1, h->counter);
    note_launch();
    unsigned long long und = 0;
    int rc = read_u64(h->counter, &und, st);
    if (rc) return rc;
    if (und == 0) break;
  }
  k_root_flags<<<gn, kT, 0, st>>>(n, state, flags);
  note_launch();
  int rc = scan_total(h, flags, ids, n, &L.n_agg, st);
  if (rc) return rc;
  k_root_ids<<<gn, kT, 0, st>>>(n, state, ids, agg2);
  note_launch();
  k_agg_join<<<gn, kT, 0, st>>>(L.g, active, agg2, L.agg);
  note_launch();
  k_agg_join<<<gn, kT, 0, st>>>(L.g, active, L.agg, agg2);
  note_launch();
  cudaMemcpyAsync(L.agg, agg2, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), st);
  k_count_unassigned<<<gn, kT, 0, st>>>(n, active, L.agg, h->counter);
  note_launch();
  unsigned long long un = 0;
  rc = read_u64(h->counter, &un, st);
  if (rc) return rc;
  if (un != 0) {
    set_last_error("AMG aggregation left %llu nodes unassigned", un);
    return FEM_CUDA_ERROR;
  }
  return FEM_OK;
}

template <int B, int K>
int tentative(fem_amg* h, int l, const double* coords, const uint8_t* con, const double* origin, const double* bn,
              double* bc, cudaStream_t st) {
  AmgLevel& L = h->L[l];
  const int64_t n = L.n, na = L.n_agg;
  int64_t* cnt = h->alloc<int64_t>(na, st);
  int64_t* aptr = h->alloc<int64_t>(na + 1, st);
  int64_t* cur = h->alloc<int64_t>(na + 1, st);
  int32_t* unsorted = h->alloc<int32_t>(n, st);
  int32_t* nodes = h->alloc<int32_t>(n, st);
  L.tval = h->alloc<float>(n * B * K, st);
  if (!cnt || !aptr || !cur || !unsorted || !nodes || !L.tval) return check_cuda("AMG tentative buffers");
  cudaMemsetAsync(cnt, 0, sizeof(int64_t) * na, st);
  cudaMemsetAsync(L.tval, 0, sizeof(float) * n * B * K, st);
  k_count_keys<<<grid_for(n, kT), kT, 0, st>>>(n, L.agg, cnt);
  note_launch();
  int64_t members = 0;
  int rc = scan_total(h, cnt, aptr, na, &members, st);
  if (rc) return rc;
  cudaMemcpyAsync(cur, aptr, sizeof(int64_t) * (na + 1), cudaMemcpyDeviceToDevice, st);
  k_fill_keys<<<grid_for(n, kT), kT, 0, st>>>(n, L.agg, cur, unsorted);
  note_launch();
  k_sort_rows<<<grid_for(na * 32, kT), kT, 0, st>>>(na, aptr, unsorted, nodes);
  note_launch();
  cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), st);
  k_tentative<B, K><<<grid_for(na, 4), 128, 0, st>>>(na, aptr, nodes, coords, con, origin, bn, L.tval, bc,
                                                     h->counter);
  note_launch();
  unsigned long long nd = 0;
  rc = read_u64(h->counter, &nd, st);
  if (rc) return rc;
  h->dropped += (int64_t)nd;
  return check_cuda("AMG tentative prolongator");
}

// Patterns of P, P^T, A P and the coarse operator of level l.
int patterns(fem_amg* h, int l, cudaStream_t st) {
  AmgLevel& L = h->L[l];
  AmgLevel& C = h->L[l + 1];
  const int64_t n = L.n, na = L.n_agg;
  const uint8_t* active = l == 0 ? h->active : nullptr;
  int64_t* cnt = h->alloc<int64_t>(std::max(n, na) + 1, st);
  L.p_ptr = h->alloc<int64_t>(n + 1, st);
  if (!cnt || !L.p_ptr) return check_cuda("AMG pattern buffers");
  const unsigned gn = grid_for(n, kT);
  k_p_rows<false><<<gn, kT, 0, st>>>(L.g, active, L.agg, cnt, nullptr, nullptr, h->status);
  note_launch();
  int rc = scan_total(h, cnt, L.p_ptr, n, &L.p_nnz, st);
  if (rc) return rc;
  L.p_col = h->alloc<int32_t>(L.p_nnz, st);
  if (!L.p_col) return check_cuda("AMG P pattern");
  k_p_rows<true><<<gn, kT, 0, st>>>(L.g, active, L.agg, nullptr, L.p_ptr, L.p_col, h->status);
  note_launch();
  {  // contribution lists of A T, in ascending neighbour per block
    L.p_row = h->alloc<int32_t>(L.p_nnz, st);
    int64_t* tcnt = h->alloc<int64_t>(L.p_nnz + 1, st);
    L.tl_ptr = h->alloc<int64_t>(L.p_nnz + 1, st);
    int64_t* tcur = h->alloc<int64_t>(L.p_nnz + 1, st);
    if (!L.p_row || !tcnt || !L.tl_ptr || !tcur) return check_cuda("AMG A T lists");
    cudaMemsetAsync(tcnt, 0, sizeof(int64_t) * (L.p_nnz + 1), st);
    k_p_lists<false><<<gn, kT, 0, st>>>(L.g, L.agg, L.p_ptr, L.p_col, tcnt, nullptr, nullptr, nullptr);
    note_launch();
    int64_t n_tl = 0;
    rc = scan_total(h, tcnt, L.tl_ptr, L.p_nnz, &n_tl, st);
    if (rc) return rc;
    L.tl_k = h->alloc<int32_t>(n_tl, st);
    if (!L.tl_k) return check_cuda("AMG A T lists");
    cudaMemcpyAsync(tcur, L.tl_ptr, sizeof(int64_t) * (L.p_nnz + 1), cudaMemcpyDeviceToDevice, st);
    k_p_lists<true><<<gn, kT, 0, st>>>(L.g, L.agg, L.p_ptr, L.p_col, nullptr, tcur, L.tl_k, L.p_row);
    note_launch();
  }
  // P^T
  L.pt_ptr = h->alloc<int64_t>(na + 1, st);
  int64_t* cur = h->alloc<int64_t>(na + 1, st);
  int32_t* unsorted = h->alloc<int32_t>(L.p_nnz, st);
  L.pt_row = h->alloc<int32_t>(L.p_nnz, st);
  L.pt_pos = h->alloc<int64_t>(L.p_nnz, st);
  if (!L.pt_ptr || !cur || !unsorted || !L.pt_row || !L.pt_pos) return check_cuda("AMG transpose buffers");
  cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (na + 1), st);
  k_count_cols<<<gn, kT, 0, st>>>(n, L.p_ptr, L.p_col, cnt);
  note_launch();
  int64_t tot = 0;
  rc = scan_total(h, cnt, L.pt_ptr, na, &tot, st);
  if (rc) return rc;
  cudaMemcpyAsync(cur, L.pt_ptr, sizeof(int64_t) * (na + 1), cudaMemcpyDeviceToDevice, st);
  k_fill_cols<<<gn, kT, 0, st>>>(n, L.p_ptr, L.p_col, cur, unsorted);
  note_launch();
  k_sort_rows<<<grid_for(na * 32, kT), kT, 0, st>>>(na, L.pt_ptr, unsorted, L.pt_row);
  note_launch();
  k_pt_pos<<<grid_for(na, kT), kT, 0, st>>>(na, L.pt_ptr, L.pt_row, L.p_ptr, L.p_col, L.pt_pos);
  note_launch();
  // A P: union of the P rows of the neighbours (rows of inactive nodes stay
  // empty: their P rows are empty and no coarse row reads them)
  L.ap_ptr = h->alloc<int64_t>(n + 1, st);
  if (!L.ap_ptr) return check_cuda("AMG AP pattern");
  k_union_rows<kMaxAPRow, false><<<gn, kT, 0, st>>>(n, active, L.g.ptr, L.g.idx, L.p_ptr, L.p_col, cnt, nullptr,
                                                     nullptr, h->status);
  note_launch();
  rc = scan_total(h, cnt, L.ap_ptr, n, &L.ap_nnz, st);
  if (rc) return rc;
  L.ap_col = h->alloc<int32_t>(L.ap_nnz, st);
  if (!L.ap_col) return check_cuda("AMG AP pattern");
  k_union_rows<kMaxAPRow, true><<<gn, kT, 0, st>>>(n, active, L.g.ptr, L.g.idx, L.p_ptr, L.p_col, nullptr,
                                                    L.ap_ptr, L.ap_col, h->status);
  note_launch();
  // coarse operator: union over the P^T row of the A P rows
  C.n = na;
  C.b = h->K;
  C.a_ptr = h->alloc<int64_t>(na + 1, st);
  if (!C.a_ptr) return check_cuda("AMG coarse pattern");
  k_union_rows<kMaxCRow, false><<<grid_for(na, kT), kT, 0, st>>>(na, nullptr, L.pt_ptr, L.pt_row, L.ap_ptr,
                                                                 L.ap_col, cnt, nullptr, nullptr, h->status);
  note_launch();
  rc = scan_total(h, cnt, C.a_ptr, na, &C.a_nnz, st);
  if (rc) return rc;
  C.a_col = h->alloc<int32_t>(C.a_nnz, st);
  if (!C.a_col) return check_cuda("AMG coarse pattern");
  k_union_rows<kMaxCRow, true><<<grid_for(na, kT), kT, 0, st>>>(na, nullptr, L.pt_ptr, L.pt_row, L.ap_ptr,
                                                                L.ap_col, nullptr, C.a_ptr, C.a_col, h->status);
  note_launch();
  C.g = Graph{na, C.a_ptr, C.a_col};
  // contribution lists of A P, in ascending neighbour per block
  {
    L.ap_row = h->alloc<int32_t>(L.ap_nnz, st);
    int64_t* wcnt = h->alloc<int64_t>(L.ap_nnz + 1, st);
    L.wl_ptr = h->alloc<int64_t>(L.ap_nnz + 1, st);
    int64_t* wcur = h->alloc<int64_t>(L.ap_nnz + 1, st);
    if (!L.ap_row || !wcnt || !L.wl_ptr || !wcur) return check_cuda("AMG A P lists");
    cudaMemsetAsync(wcnt, 0, sizeof(int64_t) * (L.ap_nnz + 1), st);
    k_ap_lists<false><<<gn, kT, 0, st>>>(L.g, active, L.p_ptr, L.p_col, L.ap_ptr, L.ap_col, wcnt, nullptr, nullptr,
                                         nullptr, nullptr);
    note_launch();
    int64_t n_wl = 0;
    rc = scan_total(h, wcnt, L.wl_ptr, L.ap_nnz, &n_wl, st);
    if (rc) return rc;
    if (n_wl >= ((int64_t)1 << 31)) {
      set_last_error("AMG: A P of level %d too large for 32-bit block indices", l);
      return FEM_BOUNDS;
    }
    L.wl_k = h->alloc<int32_t>(n_wl, st);
    L.wl_p = h->alloc<int32_t>(n_wl, st);
    if (!L.wl_k || !L.wl_p) return check_cuda("AMG A P lists");
    cudaMemcpyAsync(wcur, L.wl_ptr, sizeof(int64_t) * (L.ap_nnz + 1), cudaMemcpyDeviceToDevice, st);
    k_ap_lists<true><<<gn, kT, 0, st>>>(L.g, active, L.p_ptr, L.p_col, L.ap_ptr, L.ap_col, nullptr, wcur, L.wl_k,
                                        L.wl_p, L.ap_row);
    note_launch();
  }
  // contribution lists of the Galerkin product, in ascending fine row per block
  L.slot_row = h->alloc<int32_t>(C.a_nnz, st);
  int64_t* ccnt = h->alloc<int64_t>(C.a_nnz + 1, st);
  L.cl_ptr = h->alloc<int64_t>(C.a_nnz + 1, st);
  int64_t* ccur = h->alloc<int64_t>(C.a_nnz + 1, st);
  if (!L.slot_row || !ccnt || !L.cl_ptr || !ccur) return check_cuda("AMG Galerkin lists");
  k_slot_rows<<<grid_for(na, kT), kT, 0, st>>>(na, C.a_ptr, L.slot_row);
  note_launch();
  cudaMemsetAsync(ccnt, 0, sizeof(int64_t) * (C.a_nnz + 1), st);
  k_ac_lists<false><<<grid_for(na, 128), 128, 0, st>>>(na, L.pt_ptr, L.pt_row, L.pt_pos, L.ap_ptr, L.ap_col, C.a_ptr,
                                                       C.a_col, ccnt, nullptr, nullptr, nullptr);
  note_launch();
  int64_t n_cl = 0;
  rc = scan_total(h, ccnt, L.cl_ptr, C.a_nnz, &n_cl, st);
  if (rc) return rc;
  if (n_cl >= ((int64_t)1 << 31) || L.p_nnz >= ((int64_t)1 << 31) || L.ap_nnz >= ((int64_t)1 << 31)) {
    set_last_error("AMG: Galerkin product of level %d too large for 32-bit block indices", l);
    return FEM_BOUNDS;
  }
  L.cl_p = h->alloc<int32_t>(n_cl, st);
  L.cl_w = h->alloc<int32_t>(n_cl, st);
  if (!L.cl_p || !L.cl_w) return check_cuda("AMG Galerkin lists");
  cudaMemcpyAsync(ccur, L.cl_ptr, sizeof(int64_t) * (C.a_nnz + 1), cudaMemcpyDeviceToDevice, st);
  k_ac_lists<true><<<grid_for(na, 128), 128, 0, st>>>(na, L.pt_ptr, L.pt_row, L.pt_pos, L.ap_ptr, L.ap_col, C.a_ptr,
                                                      C.a_col, nullptr, ccur, L.cl_p, L.cl_w);
  note_launch();
  return read_status(h, st, "AMG patterns");
}

template <int B0, int K>
int create_impl(fem_amg* h, const fem_blocks* B, const double* coords, const uint8_t* con, cudaStream_t st) {
  const int64_t n0 = B->n_nod;
  h->L[0].n = n0;
  h->L[0].b = B0;
  h->L[0].g = Graph{n0, B->nbr_ptr, B->nbr};
  h->active = h->alloc<uint8_t>(n0, st);
  h->status = h->alloc<int32_t>(1, st);
  h->counter = h->alloc<unsigned long long>(1, st);
  h->ctrl = h->alloc<AmgCtrl>(1, st);
  h->lzc = h->alloc<AmgCtrl>(1, st);
  h->lz = h->alloc<double>(2 * kLanczos + 2, st);
  // per-CTA partial sums: the level-0 SpMV grid has one CTA per slice
  const int64_t n_partial = std::max<int64_t>(kPartialLen, (n0 + 31) / 32 + 1);
  h->partial = h->alloc<double>(2 * n_partial, st);
  h->s16inv = h->alloc<float>(1, st);
  h->absmax = h->alloc<unsigned int>(1, st);
  h->cyc_bar = h->alloc<CycBarrier>(1, st);
  double* origin = h->alloc<double>(3, st);
  if (!h->active || !h->status || !h->counter || !h->ctrl || !h->lzc || !h->lz || !h->partial ||
      !h->s16inv || !h->absmax || !h->cyc_bar || !origin)
    return check_cuda("AMG buffers");
  cudaMemsetAsync(h->status, 0, sizeof(int32_t), st);
  cudaMemsetAsync(h->ctrl, 0, sizeof(AmgCtrl), st);
  cudaMemsetAsync(h->lzc, 0, sizeof(AmgCtrl), st);
  k_centroid<<<1, 1024, 0, st>>>(n0, B0, coords, origin);
  note_launch();
  double* bn = nullptr;  // near-null rows of the current level (coarser levels)
  int l = 0;
  for (;; ++l) {
    AmgLevel& L = h->L[l];
    const int b = L.b;
    if (l >= 1 && L.n * b <= kCoarseMaxDof) break;
    if (l == kMaxLevels - 1) {
      set_last_error("AMG: %d levels do not reach a coarsest level of at most %d unknowns", kMaxLevels,
                     kCoarseMaxDof);
      return FEM_INVALID;
    }
    int rc = aggregate(h, l, con, st);
    if (rc) return rc;
    if (L.n_agg == 0) {
      set_last_error("AMG: no free degree of freedom to aggregate");
      return FEM_INVALID;
    }
    if (l >= 1 && L.n_agg >= L.n) {
      set_last_error("AMG: coarsening stalled at level %d (%lld block rows)", l, (long long)L.n);
      return FEM_INVALID;
    }
    double* bc = h->alloc<double>(L.n_agg * K * K, st);
    if (!bc) return check_cuda("AMG coarse near-null space");
    if (l == 0) rc = tentative<B0, K>(h, l, coords, con, origin, nullptr, bc, st);
    else rc = tentative<K, K>(h, l, nullptr, nullptr, origin, bn, bc, st);
    if (rc) return rc;
    rc = patterns(h, l, st);
    if (rc) return rc;
    bn = bc;
  }
  h->n_levels = l + 1;
  // numeric storage and vectors
  for (int k = 0; k < h->n_levels; ++k) {
    AmgLevel& L = h->L[k];
    const int64_t nv = L.n * L.b;
    if (k + 1 < h->n_levels) {
      L.p_val = h->alloc<float>(L.p_nnz * L.b * K, st);
      L.pt_val = h->alloc<__half>(L.p_nnz * L.b * K, st);
      L.p_h = h->alloc<__half>(L.p_nnz * L.b * K, st);
      L.ap_val = h->alloc<float>(L.ap_nnz * L.b * K, st);
      if (!L.p_val || !L.pt_val || !L.p_h || !L.ap_val) return check_cuda("AMG transfer storage");
    }
    if (k >= 1) {
      L.a_val = h->alloc<float>(L.a_nnz * K * K, st);
      L.dinv = h->alloc<float>(L.n * K * K, st);
      L.f = h->alloc<float>(nv, st);
      L.xb = h->alloc<float>(nv, st);
      if (!L.a_val || !L.dinv || !L.f || !L.xb) return check_cuda("AMG level storage");
    }
    L.x = h->alloc<float>(nv, st);
    L.r = h->alloc<float>(nv, st);
    L.d = h->alloc<float>(nv, st);
    L.db = h->alloc<float>(nv, st);
    if (!L.x || !L.r || !L.d || !L.db) return check_cuda("AMG vectors");
  }
  const int64_t n = n0 * B0;
  h->xlo = h->alloc<float>(n, st);
  h->rcg = h->alloc<float>(n, st);
  h->z = h->alloc<float>(n, st);
  h->p = h->alloc<float>(n, st);
  h->q = h->alloc<float>(n, st);
  AmgLevel& C = h->L[h->n_levels - 1];
  h->m_coarse = C.n * K;
  h->coarse_inv = h->alloc<float>(h->m_coarse * h->m_coarse, st);
  h->coarse_work = h->alloc<double>(2 * h->m_coarse * h->m_coarse, st);
  if (!h->xlo || !h->rcg || !h->z || !h->p || !h->q || !h->coarse_inv || !h->coarse_work)
    return check_cuda("AMG CG vectors");
  h->L[0].f = h->rcg;
  h->L[0].xb = h->z;
  cudaMemsetAsync(h->p, 0, sizeof(float) * n, st);
  return read_status(h, st, "AMG create");
}

// ---------------------------------------------------------------- numeric --
// The V-cycle vectors, block inverse and Chebyshev coefficients of level l.
OpArgs level_args(fem_amg* h, int l, AmgCtrl* ctrl) {
  AmgLevel& L = h->L[l];
  OpArgs a{};
  a.f = L.f;
  a.x = L.x;
  a.xb = L.xb;
  a.r = L.r;
  a.d = L.d;
  a.db = L.db;
  a.dinv = l == 0 ? h->dinv0 : L.dinv;
  a.theta_inv = L.theta_inv;
  a.c1 = L.c1;
  a.c2 = L.c2;
  a.partial = h->partial;
  a.ctrl = ctrl;
  a.lz = h->lz;
  a.sv16 = h->sv16;
  a.s16inv = h->s16inv;
  return a;
}

// One operator pass of level l in mode MODE (B: the level's block size).
template <int B0, int K, int MODE>
void launch_op(fem_amg* h, int l, const OpArgs& a, cudaStream_t st) {
  AmgLevel& L = h->L[l];
  if (l == 0) {
    const int64_t ns = (L.n + 31) / 32;
    const bool timed = h->ev_ready && h->ev_used < fem_amg::kTimed;
    if (timed) cudaEventRecord(h->ev[2 * h->ev_used], st);
    if (op_smoothing<MODE>() && h->sv16 && g_amg_half)
      launch_sell<B0, MODE, true>(L.n, h->sell_base, h->sell_col, h->sell_val, a, st);
    else
      launch_sell<B0, MODE, false>(L.n, h->sell_base, h->sell_col, h->sell_val, a, st);
    if constexpr (op_has_dot<MODE>()) {
      launch_chain(1, 1024, 0, st, k_dot_finish<MODE>, ns, a);
      note_launch();
    }
    if (timed) cudaEventRecord(h->ev[2 * h->ev_used++ + 1], st);
  } else {
    k_csr_op<K, MODE><<<capped(L.n, 16), kRowT, 0, st>>>(L.n, L.a_ptr, L.a_col, L.a_val, a);
  }
  note_launch();
}

// Spectral estimate of D^-1 A on level l (block size B) by kLanczos CG-Lanczos
// steps; the level's V-cycle vectors serve as scratch.
template <int B>
int lanczos_level(fem_amg* h, int l, cudaStream_t st, double* rho) {
  AmgLevel& L = h->L[l];
  const int64_t n = L.n;
  const float* dinv = l == 0 ? h->dinv0 : L.dinv;
  // scratch: r -> L.r, z -> L.d, p -> L.db, q -> L.x
  const unsigned g = capped(grid_for(n, kT), 8);
  k_lz_init<B><<<g, kT, 0, st>>>(n, dinv, L.r, L.d, L.db, h->partial, h->lzc);
  note_launch();
  OpArgs a{};
  a.p = L.db;
  a.q = L.x;
  a.partial = h->partial;
  a.ctrl = h->lzc;
  a.lz = h->lz;
  for (int j = 0; j < kLanczos; ++j) {
    bool sliced = false;
    if constexpr (B <= 3) {  // level 0 (B = dim) holds the sliced matrix
      if (l == 0) {
        const int64_t ns = (n + 31) / 32;
        launch_sell<B, kOpLzQ, false>(n, h->sell_base, h->sell_col, h->sell_val, a, st);
        note_launch();
        k_dot_finish<kOpLzQ><<<1, 1024, 0, st>>>(ns, a);
        sliced = true;
      }
    }
    if (!sliced) k_csr_op<B, kOpLzQ><<<capped(n, 16), kRowT, 0, st>>>(n, L.a_ptr, L.a_col, L.a_val, a);
    note_launch();
    k_lz_update<B><<<g, kT, 0, st>>>(n, dinv, L.r, L.d, L.x, h->partial, h->lzc, h->lz);
    note_launch();
    k_pup<<<capped(grid_for(n * B, kT), 8), kT, 0, st>>>(n * B, L.d, L.db, h->lzc);
    note_launch();
  }
  AmgCtrl hc;
  double lzh[2 * kLanczos + 2];
  if (cudaMemcpyAsync(&hc, h->lzc, sizeof(hc), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(lzh, h->lz, sizeof(lzh), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("AMG Lanczos");
  // steps whose alpha and beta are both known
  const int k = std::min(hc.lz_step, kLanczos);
  if (k < 1) {
    set_last_error("AMG: the spectral estimate of level %d broke down", l);
    return FEM_BREAKDOWN;
  }
  std::vector<double> da(k), ob(k > 1 ? k - 1 : 0);
  for (int j = 0; j < k; ++j) {
    const double al = lzh[2 * j], be_prev = j > 0 ? lzh[2 * (j - 1) + 1] : 0.0, al_prev = j > 0 ? lzh[2 * (j - 1)] : 1.0;
    da[j] = 1.0 / al + (j > 0 ? be_prev / al_prev : 0.0);
    if (j + 1 < k) ob[j] = sqrt(lzh[2 * j + 1]) / al;
  }
  *rho = tridiag_max_eig(da, ob);
  if (!(*rho > 0.0) || !std::isfinite(*rho)) {
    set_last_error("AMG: invalid spectral estimate %g at level %d", *rho, l);
    return FEM_BREAKDOWN;
  }
  return FEM_OK;
}

template <int B0, int K>
int setup_impl(fem_amg* h, const fem_matrix* A, cudaStream_t st) {
  h->sell_base = A->row_ptr;
  h->sell_col = A->col;
  h->sell_val = static_cast<const float*>(A->val);
  {
    // the V-cycle keeps its own copy of the block-Jacobi inverse, so a later
    // fem_amg_rebind to another matrix leaves the preconditioner unchanged
    const int64_t len = h->L[0].n * B0 * B0;
    if (len != h->dinv0_len) {
      if (h->dinv0_own) {
        cudaFree(h->dinv0_own);
        h->mem.erase(std::remove(h->mem.begin(), h->mem.end(), (void*)h->dinv0_own), h->mem.end());
        h->dinv0_own = nullptr;
        h->dinv0_len = 0;
      }
      h->dinv0_own = h->alloc<float>(len, st);
      if (!h->dinv0_own) return check_cuda("AMG block-Jacobi copy");
      h->dinv0_len = len;
    }
    cudaMemcpyAsync(h->dinv0_own, A->precond, sizeof(float) * len, cudaMemcpyDeviceToDevice, st);
    h->dinv0 = h->dinv0_own;
  }
  cudaMemsetAsync(h->status, 0, sizeof(int32_t), st);
  {
    // the FP16 smoothing copy, sized from the sliced layout at the first setup
    const int64_t ns = (h->L[0].n + 31) / 32;
    int64_t slots = 0;
    if (cudaMemcpyAsync(&slots, A->row_ptr + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return check_cuda("AMG setup");
    const int64_t len = slots * B0 * B0;
    if (len != h->sv16_len) {
      if (h->sv16) {
        cudaFree(h->sv16);
        h->mem.erase(std::remove(h->mem.begin(), h->mem.end(), (void*)h->sv16), h->mem.end());
        h->sv16 = nullptr;
        h->sv16_len = 0;
      }
      h->sv16 = h->alloc<__half>(len, st);
      if (!h->sv16) return check_cuda("AMG FP16 smoothing copy");
      h->sv16_len = len;
    }
    cudaMemsetAsync(h->absmax, 0, sizeof(unsigned int), st);
    k_abs_max<<<capped(grid_for(len, kT), 8), kT, 0, st>>>(len, h->sell_val, h->absmax);
    note_launch();
    k_sell_to_half<B0 * B0><<<grid_for(slots, kT), kT, 0, st>>>(slots, h->sell_val, h->absmax, h->sv16, h->s16inv);
    note_launch();
  }
  for (int l = 0; l + 1 < h->n_levels; ++l) {
    AmgLevel& L = h->L[l];
    AmgLevel& C = h->L[l + 1];
    double rho = 0.0;
    int rc = l == 0 ? lanczos_level<B0>(h, l, st, &rho) : lanczos_level<K>(h, l, st, &rho);
    if (rc) return rc;
    L.rho = rho;
    const double lo = kChebLo * rho, hi = kChebHi * rho;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    const double rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0);
    L.theta_inv = (float)(1.0 / theta);
    L.c1 = (float)(rho1 * rho0);
    L.c2 = (float)(2.0 * rho1 / delta);
    const float omega = (float)(kOmega / rho);
    if (l == 0) {
      OpView<B0, true> Av{h->sell_base, h->sell_val};
      k_p_numeric<B0, K, true><<<grid_for(L.p_nnz * 8, 256), 256, 0, st>>>(L.p_nnz, L.g, Av, h->dinv0, L.agg, L.tval,
                                                                            L.tl_ptr, L.tl_k, L.p_row, L.p_col,
                                                                            L.p_val, omega);
      note_launch();
      k_ap_numeric<B0, K, true><<<grid_for(L.ap_nnz * 8, 256), 256, 0, st>>>(L.ap_nnz, Av, L.wl_ptr, L.wl_k, L.wl_p,
                                                                            L.ap_row, L.p_val, L.ap_val);
      note_launch();
      k_ac_numeric<B0, K><<<grid_for(C.a_nnz * 32, 256), 256, 0, st>>>(C.a_nnz, L.cl_ptr, L.cl_p, L.cl_w, L.p_val,
                                                                     L.ap_val, L.slot_row, C.a_col, C.a_val);
      note_launch();
    } else {
      OpView<K, false> Av{L.a_ptr, L.a_val};
      k_p_numeric<K, K, false><<<grid_for(L.p_nnz * 8, 256), 256, 0, st>>>(L.p_nnz, L.g, Av, L.dinv, L.agg, L.tval,
                                                                            L.tl_ptr, L.tl_k, L.p_row, L.p_col,
                                                                            L.p_val, omega);
      note_launch();
      k_ap_numeric<K, K, false><<<grid_for(L.ap_nnz * 8, 256), 256, 0, st>>>(L.ap_nnz, Av, L.wl_ptr, L.wl_k, L.wl_p,
                                                                            L.ap_row, L.p_val, L.ap_val);
      note_launch();
      k_ac_numeric<K, K><<<grid_for(C.a_nnz * 32, 256), 256, 0, st>>>(C.a_nnz, L.cl_ptr, L.cl_p, L.cl_w, L.p_val,
                                                                    L.ap_val, L.slot_row, C.a_col, C.a_val);
      note_launch();
    }
    k_transfer_copies<<<grid_for(L.p_nnz * L.b * K, kT), kT, 0, st>>>(L.p_nnz, L.b * K, L.pt_pos, L.p_val, L.p_h,
                                                                      L.pt_val);
    note_launch();
    k_block_inv<K><<<grid_for(C.n, kT), kT, 0, st>>>(C.n, C.a_ptr, C.a_col, C.a_val, C.dinv, h->status);
    note_launch();
    int rc2 = check_cuda("AMG setup");
    if (rc2) return rc2;
  }
  AmgLevel& C = h->L[h->n_levels - 1];
  k_coarse_inverse<<<1, 1024, 0, st>>>(C.n, K, C.a_ptr, C.a_col, C.a_val, h->coarse_work, h->coarse_inv, h->status);
  note_launch();
  int rc = read_status(h, st, "AMG setup");
  if (rc) return rc;
  h->ready = true;
  return FEM_OK;
}

// ------------------------------------------------------------------ solve --
// The coarse part of a V-cycle, one launch per level operation: restriction
// from level 0, every coarser level's smoothing passes, the coarsest solve
// and the prolongations back to level 0.
template <int B0, int K>
void launch_coarse_levels(fem_amg* h, cudaStream_t st) {
  const int last = h->n_levels - 1;
  for (int l = 0; l < last; ++l) {
    AmgLevel& L = h->L[l];
    AmgLevel& C = h->L[l + 1];
    if (l > 0) {
      const OpArgs a = level_args(h, l, h->ctrl);
      launch_op<B0, K, kOpS1>(h, l, a, st);
      launch_op<B0, K, kOpS2>(h, l, a, st);
    }
    if (l + 1 == last) {
      if (l == 0)
        k_coarse_solve<B0, K><<<1, 1024, 0, st>>>(C.n, L.pt_ptr, L.pt_row, L.pt_val, L.r, h->coarse_inv, C.xb,
                                                  h->ctrl);
      else
        k_coarse_solve<K, K><<<1, 1024, 0, st>>>(C.n, L.pt_ptr, L.pt_row, L.pt_val, L.r, h->coarse_inv, C.xb,
                                                 h->ctrl);
    } else {
      const OpArgs c = level_args(h, l + 1, h->ctrl);
      const unsigned g = capped(C.n, 64);
      if (l == 0) k_restrict<B0, K><<<g, 128, 0, st>>>(C.n, L.pt_ptr, L.pt_row, L.pt_val, L.r, c, h->ctrl);
      else k_restrict<K, K><<<g, 128, 0, st>>>(C.n, L.pt_ptr, L.pt_row, L.pt_val, L.r, c, h->ctrl);
    }
    note_launch();
  }
  for (int l = last - 1; l >= 0; --l) {
    AmgLevel& L = h->L[l];
    AmgLevel& C = h->L[l + 1];
    if (l == 0)
      k_prolong<B0, K><<<grid_for(L.n * B0, 256), 256, 0, st>>>(L.n, L.p_ptr, L.p_col, L.p_h, C.xb, L.x, h->ctrl);
    else
      k_prolong<K, K><<<grid_for(L.n * K, 256), 256, 0, st>>>(L.n, L.p_ptr, L.p_col, L.p_h, C.xb, L.x, h->ctrl);
    note_launch();
    if (l > 0) {
      const OpArgs a = level_args(h, l, h->ctrl);
      launch_op<B0, K, kOpS3>(h, l, a, st);
      launch_op<B0, K, kOpS4>(h, l, a, st);
    }
  }
}

// The same coarse part as one cooperative launch of k_coarse_cycle.  Returns
// false when the launch is refused (the caller then runs the per-level
// kernels), after which the handle stops trying.
template <int B0, int K>
bool launch_coarse_fused(fem_amg* h, cudaStream_t st) {
  if (h->cyc_blocks < 0) return false;
  if (h->cyc_blocks == 0) {
    int dev = 0, coop = 0, occ = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_coarse_cycle<B0, K>, kCycT, 0) != cudaSuccess ||
        occ < 1) {
      cudaGetLastError();
      h->cyc_blocks = -1;
      return false;
    }
    h->cyc_blocks = std::min(occ, kCycPerSm) * sm_count();
    // small hierarchies: no more CTAs than level 1 has rows for their warps
    // (each grid barrier waits for every CTA)
    const int64_t need = (h->L[1].n + kCycT / 32 - 1) / (kCycT / 32);
    h->cyc_blocks = (int)std::max<int64_t>(std::min<int64_t>(need, h->cyc_blocks), std::min(32, h->cyc_blocks));
  }
  CycArgs ca{};
  ca.n_levels = h->n_levels;
  for (int l = 0; l < h->n_levels; ++l) {
    const AmgLevel& L = h->L[l];
    CycLevel& c = ca.L[l];
    c.n = L.n;
    c.a_ptr = L.a_ptr;
    c.a_col = L.a_col;
    c.a_val = L.a_val;
    c.dinv = l == 0 ? h->dinv0 : L.dinv;
    c.f = L.f;
    c.x = L.x;
    c.xb = L.xb;
    c.r = L.r;
    c.d = L.d;
    c.db = L.db;
    c.theta_inv = L.theta_inv;
    c.c1 = L.c1;
    c.c2 = L.c2;
    c.p_ptr = L.p_ptr;
    c.p_col = L.p_col;
    c.p_h = L.p_h;
    c.pt_ptr = L.pt_ptr;
    c.pt_row = L.pt_row;
    c.pt_val = L.pt_val;
  }
  ca.coarse_inv = h->coarse_inv;
  ca.ctrl = h->ctrl;
  ca.bar = h->cyc_bar;

  void* args[] = {&ca};
  if (cudaLaunchCooperativeKernel((const void*)k_coarse_cycle<B0, K>, dim3(h->cyc_blocks), dim3(kCycT), args, 0,
                                  st) != cudaSuccess) {
    cudaGetLastError();
    h->cyc_blocks = -1;
    return false;
  }
  note_launch();
  return true;
}

template <int B0, int K>
void launch_vcycle(fem_amg* h, cudaStream_t st) {
  const OpArgs a = level_args(h, 0, h->ctrl);
  launch_op<B0, K, kOpS1>(h, 0, a, st);
  launch_op<B0, K, kOpS2>(h, 0, a, st);
  if (h->n_levels > 1 && !(g_amg_fused && launch_coarse_fused<B0, K>(h, st))) launch_coarse_levels<B0, K>(h, st);
  launch_op<B0, K, kOpS3>(h, 0, a, st);
  launch_op<B0, K, kOpS4Dot>(h, 0, a, st);
}

template <int B0, int K>
void launch_iteration(fem_amg* h, cudaStream_t st) {
  launch_vcycle<B0, K>(h, st);
  OpArgs a{};
  a.p = h->p;
  a.q = h->q;
  a.xb = h->z;
  a.partial = h->partial;
  a.ctrl = h->ctrl;
  launch_op<B0, K, kOpQc>(h, 0, a, st);
  launch_chain(capped(grid_for(h->L[0].n, kT), 8), kT, 0, st, k_cg_update<B0>, h->L[0].n, h->xlo, h->rcg, h->p,
               h->q, h->dinv0, h->L[0].theta_inv, h->L[0].d, h->L[0].x, h->partial, h->ctrl);
  note_launch();
}

int read_ctrl(fem_amg* h, AmgCtrl* c, cudaStream_t st) {
  if (cudaMemcpyAsync(c, h->ctrl, sizeof(AmgCtrl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("AMG CG");
  return FEM_OK;
}

int status_code(int done) {
  switch (done) {
    case kConverged: return FEM_OK;
    case kMaxIter: return FEM_NOT_CONVERGED;
    case kNonFinite: return FEM_NONFINITE;
    case kBarrierTimeout: return FEM_CUDA_ERROR;
    default: return FEM_BREAKDOWN;
  }
}

int64_t op_fe_len(const fem_operator64* op) {
  int ne, d, nip;
  if (!op || etype_info(op->mesh->etype, &ne, &d, &nip) != FEM_OK) return -1;
  if (op->mesh->dof_per_node > 0) d = op->mesh->dof_per_node;
  return op->mesh->n_elem * ne * d;
}

template <int B0, int K>
int pcg_impl(fem_amg* h, const fem_matrix* A, const fem_operator64* op, const double* b, double* x, double rtol,
             double delta, int64_t max_iter, void* ws, fem_solve_info* info, cudaStream_t st) {
  const int64_t nn = h->L[0].n, n = nn * B0;
  AmgCtrl c;
  memset(&c, 0, sizeof(c));
  c.max_iter = max_iter;
  c.mixed = op ? 1 : 0;
  c.delta2 = delta * delta;
  c.rscale = 1.0;
  cudaMemcpyAsync(h->ctrl, &c, sizeof(c), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(x, 0, sizeof(double) * n, st);
  cudaMemsetAsync(h->xlo, 0, sizeof(float) * n, st);
  cudaMemsetAsync(h->p, 0, sizeof(float) * n, st);
  cudaMemsetAsync(h->q, 0, sizeof(float) * n, st);  // q carries A p: finite before the first beta = 0 update
  cudaMemsetAsync(h->cyc_bar, 0, sizeof(CycBarrier), st);  // the fused cycle's barriers count from 0 per solve
  const unsigned gv = capped(grid_for(nn, kT), 8);
  k_cg_bnorm<<<capped(grid_for(n, kT), 8), kT, 0, st>>>(n, b, rtol * rtol, h->partial, h->ctrl);
  note_launch();
  k_cg_init<B0><<<gv, kT, 0, st>>>(nn, b, h->rcg, h->dinv0, h->L[0].theta_inv, h->L[0].d, h->L[0].x, h->partial,
                                   h->ctrl);
  note_launch();
  int rc = read_ctrl(h, &c, st);
  if (rc) return rc;
  double* y64 = nullptr;
  double* fe = nullptr;
  if (op) {
    y64 = static_cast<double*>(ws);
    fe = y64 + ((n + 31) & ~int64_t(31));
  }
  constexpr int kStall = 8;
  double best = -1.0;
  int stalled = 0;
  int chunk = 2;
  h->timed_ms = 0.0;
  h->timed_n = 0;
  if (g_timing && !h->ev_ready) {
    bool ok = true;
    for (int k = 0; k < 2 * fem_amg::kTimed && ok; ++k) ok = cudaEventCreate(&h->ev[k]) == cudaSuccess;
    if (!ok) return check_cuda("AMG timing events");
    h->ev_ready = true;
  }
  const bool timing = g_timing && h->ev_ready;
  constexpr int kFinePerIter = 5;  // level-0 SpMVs per iteration: S1, S2, S3, S4, q = A p
  while (c.done == kRun) {
    if (c.replace) {
      k_cg_fold<<<grid_for(n, kT), kT, 0, st>>>(n, x, h->xlo, h->ctrl);
      note_launch();
      if (op->sell_val64) {  // one FP64 sliced SpMV over the FP64 copy of the matrix
        rc = sell_apply64(A, op->sell_val64, x, y64, st);
      } else {  // the FP64 element pass
        rc = fem_element_force(op->mesh, op->mat, x, op->con_mask, nullptr, 2, nullptr, nullptr, fe, nullptr,
                               nullptr, nullptr, st);
        if (!rc) rc = fem_gather_nodal(op->mesh, fe, nullptr, op->con_mask, 2, x, y64, nullptr, nullptr, 0, st);
      }
      if (rc) return rc;
      k_cg_replace<B0><<<gv, kT, 0, st>>>(nn, b, y64, h->rcg, h->dinv0, h->L[0].theta_inv, h->L[0].d, h->L[0].x,
                                          h->partial, h->ctrl);
      note_launch();
      rc = read_ctrl(h, &c, st);
      if (rc) return rc;
      if (c.done == kRun) {
        if (best < 0.0 || c.rr_true < 0.25 * best) {
          best = c.rr_true;
          stalled = 0;
        } else if (++stalled >= kStall) {
          set_last_error("multigrid CG stagnated at relative residual %.3e after %lld iterations: FP32 storage "
                         "cannot refine this system; use precision fp64",
                         c.bb > 0 ? sqrt(c.rr_true / c.bb) : 0.0, c.iters);
          if (info) {
            info->iterations = c.iters;
            info->replacements = c.replacements;
            info->rel_residual = c.bb > 0 ? sqrt(c.rr_true / c.bb) : 0.0;
            info->status = FEM_NOT_CONVERGED;
          }
          return FEM_NOT_CONVERGED;
        }
      }
      continue;
    }
    const long long before = c.iters;
    h->ev_used = 0;
    if (!timing) h->ev_used = fem_amg::kTimed;  // no events recorded
    for (int k = 0; k < chunk; ++k) launch_iteration<B0, K>(h, st);
    rc = check_cuda("AMG CG iteration");
    if (rc) return rc;
    rc = read_ctrl(h, &c, st);
    if (rc) return rc;
    if (timing) {
      // the launches of iterations that ran (the ones after convergence or a
      // pending replacement return at once and are not counted)
      const int active = (int)std::min<long long>(c.iters - before, chunk) * kFinePerIter;
      for (int k = 0; k < active && k < h->ev_used; ++k) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, h->ev[2 * k], h->ev[2 * k + 1]) == cudaSuccess) {
          h->timed_ms += t;
          h->timed_n += 1;
        }
      }
    }
    h->ev_used = fem_amg::kTimed;
    chunk = std::min(chunk + 1, 4);
  }
  if (op) {
    k_cg_fold<<<grid_for(n, kT), kT, 0, st>>>(n, x, h->xlo, h->ctrl);
  } else {
    k_cg_out<<<grid_for(n, kT), kT, 0, st>>>(n, h->xlo, x, h->ctrl);
  }
  note_launch();
  rc = check_cuda("AMG CG finish");
  if (rc) return rc;
  const double rel = c.bb > 0 ? (op ? sqrt(c.rr_true / c.bb) : sqrt(c.rr / c.bb) / c.rscale) : 0.0;
  if (info) {
    info->iterations = c.iters;
    info->replacements = c.replacements;
    info->rel_residual = rel;
    info->status = status_code(c.done);
    info->spmv_ms = h->timed_ms;
    info->spmv_timed = h->timed_n;
  }
  if (c.done == kBarrierTimeout)
    set_last_error("multigrid CG: a grid-barrier wait of the fused coarse cycle ran out (barrier timeout)");
  else if (c.done != kConverged)
    set_last_error("multigrid CG did not converge: %lld iterations, relative residual %.3e, code %d", c.iters, rel,
                   c.done);
  return status_code(c.done);
}

}  // namespace
}  // namespace tfg

using namespace tfg;

extern "C" {

int fem_amg_create(const fem_blocks* B, const double* coords, const uint8_t* con_mask, fem_amg** out,
                   void* stream) {
  if (!B || !coords || !out || B->n_nod <= 0 || !(B->dim >= 1 && B->dim <= 3)) {
    set_last_error("fem_amg_create: needs the node graph, coordinates and 1, 2 or 3 DOFs per node");
    return FEM_INVALID;
  }
  if (B->n_nod >= (int64_t)1 << 31) {
    set_last_error("fem_amg_create: at most 2^31 - 1 nodes");
    return FEM_BOUNDS;
  }
  cudaStream_t st = as_stream(stream);
  fem_amg* h = new fem_amg();
  h->dim = B->dim;
  // near-null space: rigid-body modes (6 in 3D, 3 in 2D) or, for one DOF per
  // node (heat conduction), the constant field
  h->K = B->dim == 3 ? 6 : (B->dim == 2 ? 3 : 1);
  const int rc = B->dim == 3   ? create_impl<3, 6>(h, B, coords, con_mask, st)
                 : B->dim == 2 ? create_impl<2, 3>(h, B, coords, con_mask, st)
                               : create_impl<1, 1>(h, B, coords, con_mask, st);
  if (rc) {
    fem_amg_destroy(h);
    *out = nullptr;
    return rc;
  }
  *out = h;
  return FEM_OK;
}

void fem_amg_destroy(fem_amg* h) {
  if (!h) return;
  if (h->ev_ready)
    for (int k = 0; k < 2 * fem_amg::kTimed; ++k) cudaEventDestroy(h->ev[k]);
  for (void* p : h->mem) cudaFree(p);
  delete h;
}

int fem_amg_setup(fem_amg* h, const fem_matrix* A, void* stream) {
  if (!h || !A || A->format != FEM_FMT_SELL_F32 || A->block != h->dim || A->n_rows != h->L[0].n || !A->precond) {
    set_last_error("fem_amg_setup: needs the FP32 sliced-block matrix (with its block-Jacobi inverse) of the "
                   "mesh the hierarchy was built on");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  h->ready = false;
  return h->dim == 3 ? setup_impl<3, 6>(h, A, st) : h->dim == 2 ? setup_impl<2, 3>(h, A, st) : setup_impl<1, 1>(h, A, st);
}

int fem_amg_rebind(fem_amg* h, const fem_matrix* A) {
  if (!h || !h->ready || !A || A->format != FEM_FMT_SELL_F32 || A->block != h->dim || A->row_ptr != h->sell_base ||
      A->col != h->sell_col) {
    set_last_error("fem_amg_rebind: needs a set-up hierarchy and an FP32 sliced matrix of the same layout");
    return FEM_INVALID;
  }
  if (!g_amg_half || !h->sv16) {
    set_last_error("fem_amg_rebind: the V-cycle would smooth on the new matrix with the old bounds; it needs the "
                   "FP16 smoothing copy");
    return FEM_INVALID;
  }
  h->sell_val = static_cast<const float*>(A->val);
  return FEM_OK;
}

size_t fem_amg_pcg_workspace_bytes(const fem_amg* h, const fem_operator64* op) {
  if (!h) return 0;
  if (!op) return 256;
  const int64_t fl = op_fe_len(op);
  if (fl < 0) return 0;
  const int64_t n = h->L[0].n * h->dim;
  return sizeof(double) * (size_t)(((n + 31) & ~int64_t(31)) + std::max<int64_t>(fl, 1)) + 256;
}

int fem_amg_pcg(fem_amg* h, const fem_matrix* A, const fem_operator64* op, const double* b, double* x, double rtol,
                double delta, int64_t max_iter, void* ws, size_t ws_bytes, fem_solve_info* info, void* stream) {
  if (!h || !h->ready) {
    set_last_error("fem_amg_pcg: the hierarchy has no numeric setup (call fem_amg_setup)");
    return FEM_INVALID;
  }
  if (!A || A->row_ptr != h->sell_base || A->val != h->sell_val) {
    set_last_error("fem_amg_pcg: the matrix differs from the one of the last fem_amg_setup or fem_amg_rebind");
    return FEM_INVALID;
  }
  if (ws_bytes < fem_amg_pcg_workspace_bytes(h, op) || (op && !ws)) {
    set_last_error("fem_amg_pcg: workspace too small");
    return FEM_INVALID;
  }
  if (!(delta > 0.0 && delta < 1.0)) {
    set_last_error("fem_amg_pcg: delta must lie in (0, 1)");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  if (h->dim == 3) return pcg_impl<3, 6>(h, A, op, b, x, rtol, delta, max_iter, ws, info, st);
  if (h->dim == 2) return pcg_impl<2, 3>(h, A, op, b, x, rtol, delta, max_iter, ws, info, st);
  return pcg_impl<1, 1>(h, A, op, b, x, rtol, delta, max_iter, ws, info, st);
}

void fem_amg_set_half_smoother(int enable) { g_amg_half = enable ? 1 : 0; }
void fem_amg_set_level0_tma(int enable) { g_amg_tma = enable ? 1 : 0; }
void fem_amg_set_pdl(int enable) { g_amg_pdl = enable ? 1 : 0; }

void fem_amg_set_fused_cycle(int enable) { g_amg_fused = enable ? 1 : 0; }

int fem_amg_levels(const fem_amg* h) { return h ? h->n_levels : 0; }

int fem_amg_level_info(const fem_amg* h, int level, fem_amg_level* out) {
  if (!h || !out || level < 0 || level >= h->n_levels) {
    set_last_error("fem_amg_level_info: no such level");
    return FEM_INVALID;
  }
  const AmgLevel& L = h->L[level];
  fem_amg_level o;
  memset(&o, 0, sizeof(o));
  o.n = L.n;
  o.block = L.b;
  o.a_nnz = L.a_nnz;
  o.a_ptr = L.a_ptr;
  o.a_col = L.a_col;
  o.a_val = L.a_val;
  o.n_agg = level + 1 < h->n_levels ? L.n_agg : 0;
  o.agg = L.agg;
  o.tval = L.tval;
  o.p_nnz = L.p_nnz;
  o.p_ptr = L.p_ptr;
  o.p_col = L.p_col;
  o.p_val = L.p_val;
  o.rho = L.rho;
  o.coarse_inv = level + 1 == h->n_levels ? h->coarse_inv : nullptr;
  o.dropped = h->dropped;
  *out = o;
  return FEM_OK;
}

int fem_copy_device(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes == 0) return FEM_OK;
  if (!dst || !src) {
    set_last_error("fem_copy_device: null pointer");
    return FEM_INVALID;
  }
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, as_stream(stream)) != cudaSuccess)
    return check_cuda("fem_copy_device");
  return FEM_OK;
}

}  // extern "C"
