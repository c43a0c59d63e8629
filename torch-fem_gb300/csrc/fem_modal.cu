// Kernels of the modal analysis (FEM.solve_modes, src/torchfem/base.py:
// 1097-1129, with the eigen-solve of src/torchfem/sparse.py:798-1011):
//  - element mass matrices of a mechanics model, the reference's
//    integrate_mass (base.py:376-396) with compute_m (solid.py:60-62,
//    planar.py:94-96): m_e = sum_ip w detJ rho t N N^T, expanded to the d
//    DOFs of each node (Kronecker product with I_d);
//  - the FP64 CSR product with a block of vectors, the operator applications
//    of the block eigensolver (LOBPCG) that replaces the reference's
//    shift-invert eigsh.
// The eigenvalue sensitivities reuse the element vector-Jacobian products
// (fem_element_vjp for K, fem_heat_mass_vjp for M).
#include "fem_common.cuh"

namespace tfg {
namespace {

// Row a of the element mass matrix of element e, a thread per (e, a).
template <int NE, int D, int NIP>
__global__ void k_mass_blocks(int64_t n_elem, int d, const double* __restrict__ detj, const double* __restrict__ w,
                              const double* __restrict__ rho, const double* __restrict__ thick,
                              const double* __restrict__ nval, double* __restrict__ me) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elem * NE) return;
  const int64_t e = t / NE;
  const int a = (int)(t % NE);
  const double c = rho[e] * (thick ? thick[e] : 1.0);
  double row[NE];
#pragma unroll
  for (int b = 0; b < NE; ++b) row[b] = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const double s = w[ip] * detj[(int64_t)ip * n_elem + e] * c * nval[ip * NE + a];
#pragma unroll
    for (int b = 0; b < NE; ++b) row[b] += s * nval[ip * NE + b];
  }
  const int64_t nd = (int64_t)NE * d;
  for (int i = 0; i < d; ++i) {
    double* out = me + (e * nd + (int64_t)a * d + i) * nd;
#pragma unroll
    for (int b = 0; b < NE; ++b)
      for (int j = 0; j < d; ++j) out[b * d + j] = i == j ? row[b] : 0.0;
  }
}

// Y[:, c0:c0+NV] = A X[:, c0:c0+NV] for an FP64 CSR matrix and row-major
// blocks X, Y [n][nv]: a warp per row, lanes over the row's entries, then
// an xor-tree sum per column (fixed order).
constexpr int kSpmmNV = 8;
__global__ void __launch_bounds__(256) k_csr_spmm(int64_t n, const int64_t* __restrict__ row_ptr,
                                                  const int32_t* __restrict__ col, const double* __restrict__ val,
                                                  int nv, int c0, const double* __restrict__ X,
                                                  double* __restrict__ Y) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const int m = min(kSpmmNV, nv - c0);
  double acc[kSpmmNV];
#pragma unroll
  for (int v = 0; v < kSpmmNV; ++v) acc[v] = 0.0;
  for (int64_t k = row_ptr[row] + lane; k < row_ptr[row + 1]; k += 32) {
    const double a = val[k];
    const double* x = X + (int64_t)col[k] * nv + c0;
#pragma unroll
    for (int v = 0; v < kSpmmNV; ++v)
      if (v < m) acc[v] = fma(a, x[v], acc[v]);
  }
#pragma unroll
  for (int v = 0; v < kSpmmNV; ++v) acc[v] = warp_sum(acc[v]);
#pragma unroll
  for (int v = 0; v < kSpmmNV; ++v)
    if (lane == v && v < m) Y[row * nv + c0 + v] = acc[v];
}

}  // namespace
}  // namespace tfg

using namespace tfg;

extern "C" {

int fem_mass_matrices(const fem_mesh* m, const double* rho, const double* nval, int d, double* me, void* stream) {
  if (!m || !rho || !nval || !me || d < 1 || d > 3 || m->n_elem < 0) {
    set_last_error("fem_mass_matrices: mesh, rho, nval and me are required and d is 1, 2 or 3");
    return FEM_INVALID;
  }
  if (m->n_elem == 0) return FEM_OK;
  cudaStream_t st = as_stream(stream);
#define TFG_BODY                                                                                            \
  {                                                                                                         \
    k_mass_blocks<NE, D, NIP><<<grid_for(m->n_elem * NE, 128), 128, 0, st>>>(m->n_elem, d, m->detj,         \
                                                                             m->weights, rho, m->thickness, \
                                                                             nval, me);                     \
    ::tfg::note_launch();                                                                                   \
  }
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_mass_matrices");
}

int fem_csr_spmm(const fem_matrix* A, int nvec, const double* X, double* Y, void* stream) {
  if (!A || A->format != FEM_FMT_CSR_F64 || A->block != 1 || A->n != A->n_rows || nvec < 1 || !X || !Y) {
    set_last_error("fem_csr_spmm: needs a scalar FP64 CSR matrix, nvec >= 1 and X, Y");
    return FEM_INVALID;
  }
  if (A->n == 0) return FEM_OK;
  cudaStream_t st = as_stream(stream);
  for (int c0 = 0; c0 < nvec; c0 += kSpmmNV) {
    k_csr_spmm<<<grid_for(A->n * 32, 256), 256, 0, st>>>(A->n, A->row_ptr, A->col,
                                                         static_cast<const double*>(A->val), nvec, c0, X, Y);
    ::tfg::note_launch();
  }
  return check_cuda("fem_csr_spmm");
}

}  // extern "C"
