// Sparsity pattern of the global stiffness matrix (FEM.__init__,
// src/torchfem/base.py:72-122), rebuilt from the node graph on the GPU.
//
// The reference forms packed keys (row << 32 | col) for every element-matrix
// entry, takes torch.unique over them plus the diagonal, and searchsorted()s
// each entry to get k_map.  For a mechanics model with d DOFs per node every
// element contributes a dense d x d block for each pair of its nodes, so the
// unique key set is exactly {(a*d+i, b*d+j) : a, b share an element} plus
// the diagonal of nodes in no element.  Building the node adjacency
// (incidence -> per-node sorted unique neighbour list) gives the same sorted
// CSR without a global sort over n_elem * (n_e d)^2 keys.
#include <stdarg.h>

#include <atomic>

#include "fem_common.cuh"

namespace tfg {

static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static thread_local char g_last_error[512] = "";

void set_last_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int check_cuda(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error("%s: %s", where, cudaGetErrorString(e));
    return FEM_CUDA_ERROR;
  }
  return FEM_OK;
}

// ---------------------------------------------------------------- scan ----
// Exclusive prefix sum of int64 counts: out[0..n] with out[n] = total.
// Three phases (tile scan, scan of tile totals, add offsets): deterministic.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                             int64_t n, int64_t* __restrict__ tile_tot) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    v[k] = (i < n) ? in[i] : 0;
    s += v[k];
  }
  // inclusive warp scan of per-thread sums
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int64_t w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
    int64_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;  // exclusive
    if (lane == kScanThreads / 32 - 1) tile_tot[blockIdx.x] = wi;
  }
  __syncthreads();
  int64_t run = warp_tot[wid] + incl - s;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

__global__ void k_scan_totals(int64_t* tile_tot, int64_t n_tiles) {
  // single block: exclusive scan in place, tile_tot[n_tiles] = grand total
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t start = 0; start < n_tiles; start += blockDim.x) {
    const int64_t i = start + threadIdx.x;
    const int64_t v = (i < n_tiles) ? tile_tot[i] : 0;
    int64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      const int nw = blockDim.x >> 5;
      int64_t w = (lane < nw) ? warp_tot[lane] : 0;
      int64_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += t;
      }
      if (lane < nw) warp_tot[lane] = wi - w;
    }
    __syncthreads();
    const int64_t carry = carry_s;
    if (i < n_tiles) tile_tot[i] = carry + warp_tot[wid] + incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = carry + warp_tot[wid] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_tot[n_tiles] = carry_s;
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ tile_tot,
                           int64_t n_tiles) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_tot[i / kScanTile];
  if (i == 0) out[n] = tile_tot[n_tiles];
}

size_t scan_workspace_bytes(int64_t n) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  return (size_t)(tiles + 1) * sizeof(int64_t);
}

// `in` and `out` must not alias.
int scan_exclusive(const int64_t* in, int64_t* out, int64_t n, int64_t* ws, cudaStream_t st) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (n > 0) {
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, ws);
    ::tfg::note_launch();
    k_scan_totals<<<1, 1024, 0, st>>>(ws, tiles);
    ::tfg::note_launch();
    k_scan_add<<<grid_for(n + 1, 256), 256, 0, st>>>(out, n, ws, tiles);
    ::tfg::note_launch();
  } else {
    cudaMemsetAsync(out, 0, sizeof(int64_t), st);
  }
  return check_cuda("scan_exclusive");
}

// ------------------------------------------------------------ incidence ----
__global__ void k_inc_count(const int32_t* __restrict__ elements, int64_t total, int64_t n_nod,
                            unsigned long long* __restrict__ cnt, int32_t* status) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int32_t a = elements[t];
  if (a < 0 || a >= n_nod) {
    flag_status(status, kStatBounds);
    return;
  }
  atomicAdd(&cnt[a], 1ull);
}

__global__ void k_inc_fill(const int32_t* __restrict__ elements, int64_t total, int64_t n_nod,
                           const int64_t* __restrict__ inc_ptr, unsigned long long* __restrict__ cur,
                           int32_t* __restrict__ inc) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int32_t a = elements[t];
  if (a < 0 || a >= n_nod) return;
  const unsigned long long pos = atomicAdd(&cur[a], 1ull);
  inc[inc_ptr[a] + (int64_t)pos] = (int32_t)t;  // code e*n_e + local
}

// Insertion sort of each node's incidence codes (ascending element, then
// local index) — the order CPU index_add_ visits a node's contributions.
__global__ void k_inc_sort(const int64_t* __restrict__ inc_ptr, int64_t n_nod, int32_t* __restrict__ inc) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nod) return;
  const int64_t s = inc_ptr[a], e = inc_ptr[a + 1];
  for (int64_t i = s + 1; i < e; ++i) {
    const int32_t v = inc[i];
    int64_t j = i - 1;
    while (j >= s && inc[j] > v) {
      inc[j + 1] = inc[j];
      --j;
    }
    inc[j + 1] = v;
  }
}

// ------------------------------------------------------------ neighbours ----
// One warp per node gathers the nodes of its incident elements into shared
// memory, marks duplicates and (fill pass) writes the distinct ids sorted.
constexpr int kNbrWarps = 4;
constexpr int kMaxCand = 1024;

template <bool kFill>
__global__ void __launch_bounds__(kNbrWarps * 32)
k_nbr(const int32_t* __restrict__ elements, int n_e, int64_t n_nod,
      const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
      int64_t* __restrict__ nbr_cnt, const int64_t* __restrict__ nbr_ptr,
      int32_t* __restrict__ nbr, int32_t* status) {
  __shared__ int32_t cand[kNbrWarps][kMaxCand];
  __shared__ unsigned char dup[kNbrWarps][kMaxCand];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t a = (int64_t)blockIdx.x * kNbrWarps + w;
  if (a >= n_nod) return;  // whole warp exits together
  const int64_t s = inc_ptr[a], e = inc_ptr[a + 1];
  const int64_t k64 = (e - s) * n_e;
  if (k64 == 0) {  // node in no element: only its diagonal
    if (lane == 0) {
      if (kFill) nbr[nbr_ptr[a]] = (int32_t)a;
      else nbr_cnt[a] = 1;
    }
    return;
  }
  if (k64 > kMaxCand) {
    if (lane == 0) {
      flag_status(status, kStatBounds);
      if (!kFill) nbr_cnt[a] = 0;
    }
    return;
  }
  const int k = (int)k64;
  int32_t* c = cand[w];
  unsigned char* d = dup[w];
  for (int i = lane; i < k; i += 32) {
    const int32_t code = inc[s + i / n_e];
    const int64_t el = code / n_e;
    c[i] = elements[el * n_e + (i % n_e)];
  }
  __syncwarp();
  int uniq = 0;
  for (int i = lane; i < k; i += 32) {
    const int32_t v = c[i];
    unsigned char dp = 0;
    for (int j = 0; j < i; ++j)
      if (c[j] == v) {
        dp = 1;
        break;
      }
    d[i] = dp;
    uniq += dp ? 0 : 1;
  }
  __syncwarp();
  uniq = warp_sum(uniq);
  if (!kFill) {
    if (lane == 0) nbr_cnt[a] = uniq;
    return;
  }
  const int64_t base = nbr_ptr[a];
  for (int i = lane; i < k; i += 32) {
    if (d[i]) continue;
    const int32_t v = c[i];
    int pos = 0;
    for (int j = 0; j < k; ++j) pos += (!d[j] && c[j] < v) ? 1 : 0;
    nbr[base + pos] = v;
  }
}

__device__ __forceinline__ int64_t find_sorted(const int32_t* __restrict__ list, int64_t n, int32_t v) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (list[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && list[lo] == v) ? lo : -1;
}

// ------------------------------------------------------------ scalar CSR ----
__global__ void k_row_len(const int64_t* __restrict__ nbr_ptr, const int64_t* __restrict__ inc_ptr,
                          int64_t n_nod, int d, int64_t* __restrict__ len) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nod) return;
  const bool orphan = inc_ptr[a + 1] == inc_ptr[a];
  const int64_t deg = nbr_ptr[a + 1] - nbr_ptr[a];
  for (int i = 0; i < d; ++i) len[a * d + i] = orphan ? 1 : deg * d;
}

__global__ void k_csr_cols(const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                           const int64_t* __restrict__ inc_ptr, int64_t n_nod, int d,
                           const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col,
                           int64_t* __restrict__ diag_map) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_nod * d) return;
  const int64_t a = t / d;
  const int i = (int)(t % d);
  const int64_t base = row_ptr[t];
  if (inc_ptr[a + 1] == inc_ptr[a]) {
    col[base] = (int32_t)t;
    diag_map[t] = base;
    return;
  }
  const int64_t s = nbr_ptr[a], deg = nbr_ptr[a + 1] - s;
  for (int64_t k = 0; k < deg; ++k) {
    const int32_t b = nbr[s + k];
    for (int j = 0; j < d; ++j) col[base + k * d + j] = b * d + j;
    if (b == a) diag_map[t] = base + k * d + i;
  }
}

__global__ void k_kmap(const int32_t* __restrict__ elements, int64_t n_elem, int n_e, int d,
                       const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                       const int64_t* __restrict__ row_ptr, int64_t* __restrict__ k_map,
                       int32_t* status) {
  // one thread per (e, la, lb)
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nn = (int64_t)n_e * n_e;
  if (t >= n_elem * nn) return;
  const int64_t e = t / nn;
  const int la = (int)((t % nn) / n_e), lb = (int)(t % n_e);
  const int32_t a = elements[e * n_e + la], b = elements[e * n_e + lb];
  const int64_t s = nbr_ptr[a];
  const int64_t k = find_sorted(nbr + s, nbr_ptr[a + 1] - s, b);
  if (k < 0) {
    flag_status(status, kStatBounds);
    return;
  }
  const int64_t nd = (int64_t)n_e * d;
  for (int i = 0; i < d; ++i) {
    const int64_t slot0 = row_ptr[(int64_t)a * d + i] + k * d;
    const int64_t out0 = e * nd * nd + (int64_t)(la * d + i) * nd + (int64_t)lb * d;
    for (int j = 0; j < d; ++j) k_map[out0 + j] = slot0 + j;
  }
}

// ------------------------------------------------------------ blocks ----
__global__ void k_blk_count(const int32_t* __restrict__ elements, int64_t n_elem, int n_e,
                            const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                            unsigned long long* __restrict__ bcnt, int32_t* status) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nn = (int64_t)n_e * n_e;
  if (t >= n_elem * nn) return;
  const int64_t e = t / nn;
  const int la = (int)((t % nn) / n_e), lb = (int)(t % n_e);
  const int32_t a = elements[e * n_e + la], b = elements[e * n_e + lb];
  const int64_t s = nbr_ptr[a];
  const int64_t k = find_sorted(nbr + s, nbr_ptr[a + 1] - s, b);
  if (k < 0) {
    flag_status(status, kStatBounds);
    return;
  }
  atomicAdd(&bcnt[s + k], 1ull);
}

__global__ void k_blk_rows(const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                           int64_t n_nod, int32_t* __restrict__ blk_row, int64_t* __restrict__ diag_blk) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nod) return;
  const int64_t s = nbr_ptr[a], e = nbr_ptr[a + 1];
  for (int64_t k = s; k < e; ++k) {
    blk_row[k] = (int32_t)a;
    if (nbr[k] == a) diag_blk[a] = k;
  }
}

// Thread per row node: walks its incidences in ascending (element, local)
// order, so every block list comes out in the serial index_add_ order.
__global__ void k_blk_fill(const int32_t* __restrict__ elements, int n_e, int64_t n_nod,
                           const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                           const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                           const int64_t* __restrict__ blk_ptr, int64_t* __restrict__ cursor,
                           int32_t* __restrict__ contrib) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nod) return;
  const int64_t s = nbr_ptr[a], deg = nbr_ptr[a + 1] - s;
  for (int64_t q = inc_ptr[a]; q < inc_ptr[a + 1]; ++q) {
    const int32_t code = inc[q];
    const int64_t e = code / n_e;
    for (int lb = 0; lb < n_e; ++lb) {
      const int32_t b = elements[e * n_e + lb];
      const int64_t k = find_sorted(nbr + s, deg, b);
      if (k < 0) continue;
      const int64_t blk = s + k;
      const int64_t pos = blk_ptr[blk] + cursor[blk];
      cursor[blk] += 1;
      contrib[pos] = (int32_t)(((int64_t)code) * n_e + lb);
    }
  }
}

}  // namespace tfg

using namespace tfg;

extern "C" {

const char* fem_last_error(void) { return tfg::g_last_error; }
int fem_abi_version(void) { return FEM_ABI_VERSION; }
int64_t fem_launch_count(void) { return tfg::g_launches.load(std::memory_order_relaxed); }

static int64_t pattern_count_len(int64_t n_nod, int64_t n_elem, int n_e) {
  const int64_t nb_bound = n_elem * (int64_t)n_e * n_e + n_nod;  // >= n_blocks
  const int64_t dof_bound = n_nod * 8;                             // >= n_dofs
  return nb_bound > dof_bound ? nb_bound : dof_bound;
}

size_t fem_pattern_workspace_bytes(int64_t n_nod, int64_t n_elem, int n_e) {
  const int64_t m = pattern_count_len(n_nod, n_elem, n_e);
  return (size_t)m * sizeof(int64_t) + scan_workspace_bytes(m);
}

static int check_ws(size_t have, size_t need, const char* where) {
  if (have < need) {
    set_last_error("%s: workspace of %zu bytes, %zu needed", where, have, need);
    return FEM_INVALID;
  }
  return FEM_OK;
}

int fem_pattern_graph_count(const int32_t* elements, int64_t n_elem, int n_e, int64_t n_nod,
                            int64_t* inc_ptr, int32_t* inc, int64_t* nbr_ptr, int64_t* n_blocks,
                            void* ws, size_t ws_bytes, int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (n_e <= 0 || n_elem < 0 || n_nod <= 0) {
    set_last_error("fem_pattern_graph_count: bad sizes");
    return FEM_INVALID;
  }
  if (n_elem * (int64_t)n_e >= (int64_t)INT32_MAX || n_elem * (int64_t)n_e * n_e >= (int64_t)INT32_MAX) {
    set_last_error("fem_pattern_graph_count: n_elem * n_e^2 exceeds int32 contributor codes");
    return FEM_BOUNDS;
  }
  int rc = check_ws(ws_bytes, fem_pattern_workspace_bytes(n_nod, n_elem, n_e), "fem_pattern_graph_count");
  if (rc) return rc;
  int64_t* cnt = reinterpret_cast<int64_t*>(ws);
  int64_t* scan_ws = cnt + pattern_count_len(n_nod, n_elem, n_e);
  const int64_t total = n_elem * n_e;
  cudaMemsetAsync(cnt, 0, n_nod * sizeof(int64_t), st);
  k_inc_count<<<grid_for(total, 256), 256, 0, st>>>(elements, total, n_nod,
                                                    reinterpret_cast<unsigned long long*>(cnt), status);
                                                    ::tfg::note_launch();
  rc = scan_exclusive(cnt, inc_ptr, n_nod, scan_ws, st);
  if (rc) return rc;
  cudaMemsetAsync(cnt, 0, n_nod * sizeof(int64_t), st);
  k_inc_fill<<<grid_for(total, 256), 256, 0, st>>>(elements, total, n_nod, inc_ptr,
                                                   reinterpret_cast<unsigned long long*>(cnt), inc);
                                                   ::tfg::note_launch();
  k_inc_sort<<<grid_for(n_nod, 128), 128, 0, st>>>(inc_ptr, n_nod, inc);
  ::tfg::note_launch();
  k_nbr<false><<<grid_for(n_nod, kNbrWarps), kNbrWarps * 32, 0, st>>>(
      elements, n_e, n_nod, inc_ptr, inc, cnt, nullptr, nullptr, status);
      ::tfg::note_launch();
  rc = scan_exclusive(cnt, nbr_ptr, n_nod, scan_ws, st);
  if (rc) return rc;
  TFG_CHECK_LAUNCH("fem_pattern_graph_count");
  if (cudaMemcpyAsync(n_blocks, nbr_ptr + n_nod, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("fem_pattern_graph_count sync");
  return FEM_OK;
}

int fem_pattern_graph_fill(const int32_t* elements, int64_t n_elem, int n_e, int64_t n_nod,
                           const int64_t* inc_ptr, const int32_t* inc, const int64_t* nbr_ptr,
                           int32_t* nbr, int32_t* status, void* stream) {
  (void)n_elem;
  cudaStream_t st = as_stream(stream);
  k_nbr<true><<<grid_for(n_nod, kNbrWarps), kNbrWarps * 32, 0, st>>>(
      elements, n_e, n_nod, inc_ptr, inc, nullptr, nbr_ptr, nbr, status);
      ::tfg::note_launch();
  return check_cuda("fem_pattern_graph_fill");
}

int fem_pattern_csr_rows(const int64_t* nbr_ptr, int64_t n_nod, int dof_per_node,
                         const int64_t* inc_ptr, int64_t* row_ptr, int64_t* nnz, void* ws,
                         size_t ws_bytes, void* stream) {
  cudaStream_t st = as_stream(stream);
  const int64_t n = n_nod * dof_per_node;
  const size_t need = (size_t)n * sizeof(int64_t) + scan_workspace_bytes(n);
  int rc = check_ws(ws_bytes, need, "fem_pattern_csr_rows");
  if (rc) return rc;
  int64_t* len = reinterpret_cast<int64_t*>(ws);
  k_row_len<<<grid_for(n_nod, 256), 256, 0, st>>>(nbr_ptr, inc_ptr, n_nod, dof_per_node, len);
  ::tfg::note_launch();
  rc = scan_exclusive(len, row_ptr, n, len + n, st);
  if (rc) return rc;
  if (cudaMemcpyAsync(nnz, row_ptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return check_cuda("fem_pattern_csr_rows sync");
  return check_cuda("fem_pattern_csr_rows");
}

int fem_pattern_csr_cols(const int64_t* nbr_ptr, const int32_t* nbr, int64_t n_nod, int dof_per_node,
                         const int64_t* inc_ptr, const int64_t* row_ptr, int32_t* col,
                         int64_t* diag_map, void* stream) {
  cudaStream_t st = as_stream(stream);
  const int64_t n = n_nod * dof_per_node;
  k_csr_cols<<<grid_for(n, 128), 128, 0, st>>>(nbr_ptr, nbr, inc_ptr, n_nod, dof_per_node, row_ptr,
                                               col, diag_map);
                                               ::tfg::note_launch();
  return check_cuda("fem_pattern_csr_cols");
}

int fem_pattern_kmap(const int32_t* elements, int64_t n_elem, int n_e, int dof_per_node,
                     const int64_t* nbr_ptr, const int32_t* nbr, const int64_t* row_ptr,
                     int64_t* k_map, int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  const int64_t t = n_elem * n_e * n_e;
  k_kmap<<<grid_for(t, 256), 256, 0, st>>>(elements, n_elem, n_e, dof_per_node, nbr_ptr, nbr,
                                           row_ptr, k_map, status);
                                           ::tfg::note_launch();
  return check_cuda("fem_pattern_kmap");
}

int fem_pattern_blocks(const int32_t* elements, int64_t n_elem, int n_e, int64_t n_nod,
                       const int64_t* inc_ptr, const int32_t* inc, const int64_t* nbr_ptr,
                       const int32_t* nbr, int64_t n_blocks, int64_t* blk_ptr, int32_t* contrib,
                       int32_t* blk_row, int64_t* diag_blk, void* ws, size_t ws_bytes,
                       int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  const size_t need = (size_t)n_blocks * sizeof(int64_t) + scan_workspace_bytes(n_blocks);
  int rc = check_ws(ws_bytes, need, "fem_pattern_blocks");
  if (rc) return rc;
  int64_t* bcnt = reinterpret_cast<int64_t*>(ws);
  const int64_t t = n_elem * n_e * n_e;
  cudaMemsetAsync(bcnt, 0, n_blocks * sizeof(int64_t), st);
  k_blk_count<<<grid_for(t, 256), 256, 0, st>>>(elements, n_elem, n_e, nbr_ptr, nbr,
                                                reinterpret_cast<unsigned long long*>(bcnt), status);
                                                ::tfg::note_launch();
  rc = scan_exclusive(bcnt, blk_ptr, n_blocks, bcnt + n_blocks, st);
  if (rc) return rc;
  k_blk_rows<<<grid_for(n_nod, 256), 256, 0, st>>>(nbr_ptr, nbr, n_nod, blk_row, diag_blk);
  ::tfg::note_launch();
  cudaMemsetAsync(bcnt, 0, n_blocks * sizeof(int64_t), st);
  k_blk_fill<<<grid_for(n_nod, 128), 128, 0, st>>>(elements, n_e, n_nod, inc_ptr, inc, nbr_ptr, nbr,
                                                   blk_ptr, bcnt, contrib);
                                                   ::tfg::note_launch();
  return check_cuda("fem_pattern_blocks");
}

}  // extern "C"
