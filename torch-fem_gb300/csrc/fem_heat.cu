// Heat conduction, one temperature DOF per node: Gauss-point integration of
// the conductivity matrix, the nodal heat fluxes and their vector-Jacobian
// product, and the capacity (mass) matrix.  Replaces Heat.integrate_material
// (src/torchfem/base.py:1177-1286) with the SolidHeat / PlanarHeat
// compute_k / compute_f (solid.py:52-58, planar.py:86-92) and
// FEM.integrate_mass (base.py:376-396) with compute_m (solid.py:60-62,
// planar.py:94-96), for the Fourier law of the conductivity materials
// (materials/conductivity.py: flux_new = flux + kappa (grad_inc - de0),
// tangent kappa).
//
// Layouts (device):
//   bt     [nip][n_elem][n_e][dim]   physical gradients (fem_geometry)
//   kappa  [n_elem][dim][dim]        conductivity per element
//   flux   [nip][n_elem][dim]        heat flux per point (the reference's [1, dim])
//   ke, me [n_elem][n_e][n_e]
#include "fem_common.cuh"

namespace tfg {

namespace {

template <int NE>
__device__ __forceinline__ void load_temps(const double* __restrict__ v, const int32_t* __restrict__ conn,
                                           const uint8_t* __restrict__ con_mask,
                                           const double* __restrict__ con_values, int con_mode, double (&t)[NE]) {
#pragma unroll
  for (int a = 0; a < NE; ++a) {
    const int64_t n = conn[a];
    double x = v[n];
    if (con_mode != 0 && con_mask[n]) x = (con_mode == 1) ? con_values[n] : 0.0;
    t[a] = x;
  }
}

// Thread per (element, node row a): K_ab = sum_ip w detJ t B_a^T kappa B_b.
template <int NE, int D, int NIP, typename T>
__global__ void k_heat_stiffness(int64_t n_elem, const double* __restrict__ bt, const double* __restrict__ detj,
                                 const double* __restrict__ w, const double* __restrict__ kappa,
                                 const double* __restrict__ thick, T* __restrict__ ke) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elem * NE) return;
  const int64_t e = t / NE;
  const int a = (int)(t % NE);
  double kap[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) kap[i][j] = kappa[(e * D + i) * D + j];
  const double th = thick ? thick[e] : 1.0;
  double row[NE];
#pragma unroll
  for (int b = 0; b < NE; ++b) row[b] = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const double* B = bt + ((int64_t)ip * n_elem + e) * NE * D;
    const double wj = w[ip] * detj[(int64_t)ip * n_elem + e] * th;
    double kb[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) s += B[a * D + i] * kap[i][j];
      kb[j] = s * wj;
    }
#pragma unroll
    for (int b = 0; b < NE; ++b) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) s += kb[j] * B[b * D + j];
      row[b] += s;
    }
  }
#pragma unroll
  for (int b = 0; b < NE; ++b) ke[(e * NE + a) * NE + b] = (T)row[b];
}

// Thread per element: gradient increment g = B v, flux = flux_prev +
// kappa (g - de0), f_a = sum_ip w detJ t B_a . flux.
template <int NE, int D, int NIP>
__global__ void k_heat_force(int64_t n_elem, const double* __restrict__ bt, const double* __restrict__ detj,
                             const double* __restrict__ w, const int32_t* __restrict__ elements,
                             const double* __restrict__ kappa, const double* __restrict__ thick,
                             const double* __restrict__ v, const uint8_t* __restrict__ con_mask,
                             const double* __restrict__ con_values, int con_mode,
                             const double* __restrict__ flux_prev, const double* __restrict__ de0,
                             double* __restrict__ fe, double* __restrict__ flux_out, double* __restrict__ hgrad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  double tv[NE];
  load_temps<NE>(v, elements + e * NE, con_mask, con_values, con_mode, tv);
  double kap[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) kap[i][j] = kappa[(e * D + i) * D + j];
  double e0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e0[j] = de0 ? de0[e * D + j] : 0.0;
  const double th = thick ? thick[e] : 1.0;
  double f[NE];
#pragma unroll
  for (int a = 0; a < NE; ++a) f[a] = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const int64_t pe = (int64_t)ip * n_elem + e;
    const double* B = bt + pe * NE * D;
    const double wj = w[ip] * detj[pe] * th;
    double g[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < NE; ++a) s += B[a * D + i] * tv[a];
      g[i] = s;
    }
    double q[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double s = flux_prev ? flux_prev[pe * D + i] : 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) s += kap[i][j] * (g[j] - e0[j]);
      q[i] = s;
    }
    if (flux_out)
#pragma unroll
      for (int i = 0; i < D; ++i) flux_out[pe * D + i] = q[i];
    if (hgrad)
#pragma unroll
      for (int i = 0; i < D; ++i) hgrad[pe * D + i] = g[i];
#pragma unroll
    for (int a = 0; a < NE; ++a) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) s += B[a * D + i] * q[i];
      f[a] += wj * s;
    }
  }
#pragma unroll
  for (int a = 0; a < NE; ++a) fe[e * NE + a] = f[a];
}

// Thread per element: cotangents of (assembled heat fluxes g, point fluxes
// gflux, gradient increments ghg) pulled back to flux_prev, kappa, thickness,
// de0 and the element temperatures.
template <int NE, int D, int NIP>
__global__ void k_heat_vjp(int64_t n_elem, const double* __restrict__ bt, const double* __restrict__ detj,
                           const double* __restrict__ w, const int32_t* __restrict__ elements,
                           const double* __restrict__ kappa, const double* __restrict__ thick,
                           const double* __restrict__ v, const uint8_t* __restrict__ con_mask,
                           const double* __restrict__ con_values, int con_mode, const double* __restrict__ flux_prev,
                           const double* __restrict__ de0, const double* __restrict__ g,
                           const double* __restrict__ gflux, const double* __restrict__ ghg,
                           double* __restrict__ gflux_prev, double* __restrict__ gkappa, double* __restrict__ gthick,
                           double* __restrict__ gde0, double* __restrict__ gve) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int32_t* conn = elements + e * NE;
  double tv[NE], ga[NE];
  load_temps<NE>(v, conn, con_mask, con_values, con_mode, tv);
#pragma unroll
  for (int a = 0; a < NE; ++a) ga[a] = g ? g[conn[a]] : 0.0;
  double kap[D][D], gk[D][D], e0[D], ge0[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    e0[i] = de0 ? de0[e * D + i] : 0.0;
    ge0[i] = 0.0;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      kap[i][j] = kappa[(e * D + i) * D + j];
      gk[i][j] = 0.0;
    }
  }
  const double th = thick ? thick[e] : 1.0;
  double gt = 0.0, gv[NE];
#pragma unroll
  for (int a = 0; a < NE; ++a) gv[a] = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const int64_t pe = (int64_t)ip * n_elem + e;
    const double* B = bt + pe * NE * D;
    const double w0 = w[ip] * detj[pe];
    double gr[D], q[D], phi[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double s = 0.0, c = 0.0;
#pragma unroll
      for (int a = 0; a < NE; ++a) {
        s += B[a * D + i] * tv[a];
        c += B[a * D + i] * ga[a];
      }
      gr[i] = s;
      phi[i] = w0 * th * c + (gflux ? gflux[pe * D + i] : 0.0);
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double s = flux_prev ? flux_prev[pe * D + i] : 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) s += kap[i][j] * (gr[j] - e0[j]);
      q[i] = s;
    }
    if (gflux_prev)
#pragma unroll
      for (int i = 0; i < D; ++i) gflux_prev[pe * D + i] = phi[i];
    double gg[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        s += phi[i] * kap[i][j];
        gk[i][j] += phi[i] * (gr[j] - e0[j]);
      }
      ge0[j] -= s;
      gg[j] = s + (ghg ? ghg[pe * D + j] : 0.0);
    }
#pragma unroll
    for (int a = 0; a < NE; ++a) {
      double s = 0.0, c = 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) {
        s += B[a * D + j] * gg[j];
        c += B[a * D + j] * q[j];
      }
      gv[a] += s;
      gt += w0 * ga[a] * c;
    }
  }
  if (gkappa)
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) gkappa[(e * D + i) * D + j] = gk[i][j];
  if (gthick) gthick[e] = gt;
  if (gde0)
#pragma unroll
    for (int j = 0; j < D; ++j) gde0[e * D + j] = ge0[j];
  if (gve)
#pragma unroll
    for (int a = 0; a < NE; ++a) gve[e * NE + a] = gv[a];
}

// Thread per (element, node row a): M_ab = sum_ip w detJ t rho N_a N_b.
template <int NE, int D, int NIP, typename T>
__global__ void k_heat_mass(int64_t n_elem, const double* __restrict__ detj, const double* __restrict__ w,
                            const double* __restrict__ rho, const double* __restrict__ thick,
                            const double* __restrict__ nval, T* __restrict__ me) {
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
#pragma unroll
  for (int b = 0; b < NE; ++b) me[(e * NE + a) * NE + b] = (T)row[b];
}

// Capacity vector-Jacobian product, a thread per element:
// out_e = sum_ip w detJ (N . a_e)(N . b_e), i.e. a_e^T m_e b_e / (rho_e t_e)
// for the capacity matrix m_e of k_heat_mass.
template <int NE, int D, int NIP>
__global__ void k_heat_mass_vjp(int64_t n_elem, const int32_t* __restrict__ conn, const double* __restrict__ detj,
                                const double* __restrict__ w, const double* __restrict__ nval,
                                const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  double av[NE], bv[NE];
#pragma unroll
  for (int k = 0; k < NE; ++k) {
    const int64_t nd = conn[e * NE + k];
    av[k] = a[nd];
    bv[k] = b[nd];
  }
  double s = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    double na = 0.0, nb = 0.0;
#pragma unroll
    for (int k = 0; k < NE; ++k) {
      na += nval[ip * NE + k] * av[k];
      nb += nval[ip * NE + k] * bv[k];
    }
    s += w[ip] * detj[(int64_t)ip * n_elem + e] * na * nb;
  }
  out[e] = s;
}

// out = a x + b y over the stored entries of two matrices of one pattern.
__global__ void k_csr_combine(int64_t nnz, double a, const double* __restrict__ x, double b,
                              const double* __restrict__ y, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nnz) out[i] = a * x[i] + b * y[i];
}

// Crank-Nicolson residual of one time step, a row per thread:
// res = M du + half_dt (f_old + f_int + f_ext), zero on constrained rows, and
// the per-CTA partial sums of res^2 (fixed order).
constexpr int kCnThreads = 256;
__global__ void __launch_bounds__(kCnThreads)
    k_cn_residual(int64_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                  const double* __restrict__ val, const double* __restrict__ du, const double* __restrict__ f_old,
                  const double* __restrict__ f_int, const double* __restrict__ f_ext, double half_dt,
                  const uint8_t* __restrict__ con_mask, double* __restrict__ res, double* __restrict__ partial) {
  __shared__ double red[32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double r = 0.0;
  if (i < n) {
    if (!(con_mask && con_mask[i])) {
      double s = 0.0;
      for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) s += val[k] * du[col[k]];
      const double fo = f_old ? f_old[i] : 0.0;
      const double fx = f_ext ? f_ext[i] : 0.0;
      r = s + half_dt * (fo + f_int[i] + fx);
    }
    res[i] = r;
  }
  const double t = block_sum(r * r, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void k_cn_sum(const double* __restrict__ partial, int n, double* __restrict__ sumsq) {
  __shared__ double red[32];
  const double t = sum_partials(partial, n, 1, 0, red);
  if (threadIdx.x == 0) *sumsq = t;
}

int check_heat_mesh(const fem_mesh* m, const char* what) {
  if (!m || !m->bt || !m->detj || !m->weights || !m->elements) {
    set_last_error("%s: the mesh needs its geometry (fem_geometry)", what);
    return FEM_INVALID;
  }
  return FEM_OK;
}

}  // namespace
}  // namespace tfg

using namespace tfg;

extern "C" {

int fem_heat_stiffness(const fem_mesh* m, const double* kappa, int out_dtype, void* ke, int32_t* status,
                       void* stream) {
  (void)status;
  int rc = check_heat_mesh(m, "fem_heat_stiffness");
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
#define TFG_BODY                                                                                         \
  {                                                                                                      \
    const unsigned g = grid_for(m->n_elem * NE, 128);                                                    \
    if (out_dtype == FEM_F32)                                                                            \
      k_heat_stiffness<NE, D, NIP, float><<<g, 128, 0, st>>>(m->n_elem, m->bt, m->detj, m->weights, kappa, \
                                                             m->thickness, static_cast<float*>(ke));      \
    else                                                                                                 \
      k_heat_stiffness<NE, D, NIP, double><<<g, 128, 0, st>>>(m->n_elem, m->bt, m->detj, m->weights, kappa, \
                                                              m->thickness, static_cast<double*>(ke));    \
    ::tfg::note_launch();                                                                                \
  }
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_heat_stiffness");
}

int fem_heat_force(const fem_mesh* m, const double* kappa, const double* v, const uint8_t* con_mask,
                   const double* con_values, int con_mode, const double* flux_prev, const double* de0, double* fe,
                   double* flux, double* hgrad, int32_t* status, void* stream) {
  (void)status;
  int rc = check_heat_mesh(m, "fem_heat_force");
  if (rc) return rc;
  if (con_mode != 0 && !con_mask) {
    set_last_error("fem_heat_force: con_mode needs con_mask");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
#define TFG_BODY                                                                                        \
  {                                                                                                     \
    k_heat_force<NE, D, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                 \
        m->n_elem, m->bt, m->detj, m->weights, m->elements, kappa, m->thickness, v, con_mask, con_values, \
        con_mode, flux_prev, de0, fe, flux, hgrad);                                                     \
    ::tfg::note_launch();                                                                               \
  }
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_heat_force");
}

int fem_heat_vjp(const fem_mesh* m, const double* kappa, const double* v, const uint8_t* con_mask,
                 const double* con_values, int con_mode, const double* flux_prev, const double* de0,
                 const double* g, const double* gflux, const double* ghgrad, double* gflux_prev, double* gkappa,
                 double* gthick, double* gde0, double* gve, void* stream) {
  int rc = check_heat_mesh(m, "fem_heat_vjp");
  if (rc) return rc;
  if (con_mode != 0 && !con_mask) {
    set_last_error("fem_heat_vjp: con_mode needs con_mask");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
#define TFG_BODY                                                                                        \
  {                                                                                                     \
    k_heat_vjp<NE, D, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                   \
        m->n_elem, m->bt, m->detj, m->weights, m->elements, kappa, m->thickness, v, con_mask, con_values, \
        con_mode, flux_prev, de0, g, gflux, ghgrad, gflux_prev, gkappa, gthick, gde0, gve);              \
    ::tfg::note_launch();                                                                               \
  }
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_heat_vjp");
}

int fem_heat_mass(const fem_mesh* m, const double* rho, const double* nval, int out_dtype, void* me,
                  int32_t* status, void* stream) {
  (void)status;
  int rc = check_heat_mesh(m, "fem_heat_mass");
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
#define TFG_BODY                                                                                       \
  {                                                                                                    \
    const unsigned g = grid_for(m->n_elem * NE, 128);                                                  \
    if (out_dtype == FEM_F32)                                                                          \
      k_heat_mass<NE, D, NIP, float><<<g, 128, 0, st>>>(m->n_elem, m->detj, m->weights, rho, m->thickness, \
                                                        nval, static_cast<float*>(me));                \
    else                                                                                               \
      k_heat_mass<NE, D, NIP, double><<<g, 128, 0, st>>>(m->n_elem, m->detj, m->weights, rho,          \
                                                         m->thickness, nval, static_cast<double*>(me)); \
    ::tfg::note_launch();                                                                              \
  }
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_heat_mass");
}

int fem_heat_mass_vjp(const fem_mesh* m, const double* nval, const double* a, const double* b, double* out,
                      void* stream) {
  int rc = check_heat_mesh(m, "fem_heat_mass_vjp");
  if (rc) return rc;
  if (!nval || !a || !b || !out) {
    set_last_error("fem_heat_mass_vjp: nval, a, b and out are required");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
#define TFG_BODY                                                                                         \
  {                                                                                                      \
    k_heat_mass_vjp<NE, D, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(m->n_elem, m->elements, m->detj, \
                                                                         m->weights, nval, a, b, out);  \
    ::tfg::note_launch();                                                                                \
  }
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_heat_mass_vjp");
}

int fem_csr_combine(int64_t nnz, double a, const double* x, double b, const double* y, double* out,
                    void* stream) {
  if (nnz <= 0) return FEM_OK;
  k_csr_combine<<<grid_for(nnz, 256), 256, 0, as_stream(stream)>>>(nnz, a, x, b, y, out);
  ::tfg::note_launch();
  return check_cuda("fem_csr_combine");
}

size_t fem_heat_cn_workspace_bytes(int64_t n) { return (size_t)(grid_for(n, kCnThreads) + 1) * sizeof(double); }

int fem_heat_cn_residual(const fem_matrix* M, const double* du, const double* f_old, const double* f_int,
                         const double* f_ext, double half_dt, const uint8_t* con_mask, double* res, double* sumsq,
                         void* ws, size_t ws_bytes, void* stream) {
  if (!M || M->format != FEM_FMT_CSR_F64 || M->block != 1 || M->n != M->n_rows) {
    set_last_error("fem_heat_cn_residual: the capacity matrix must be scalar FP64 CSR");
    return FEM_INVALID;
  }
  if (!du || !f_int || !res || !sumsq) {
    set_last_error("fem_heat_cn_residual: du, f_int, res and sumsq are required");
    return FEM_INVALID;
  }
  if (ws_bytes < fem_heat_cn_workspace_bytes(M->n)) {
    set_last_error("fem_heat_cn_residual: workspace too small");
    return FEM_INVALID;
  }
  cudaStream_t st = as_stream(stream);
  const unsigned g = grid_for(M->n, kCnThreads);
  double* partial = static_cast<double*>(ws);
  k_cn_residual<<<g, kCnThreads, 0, st>>>(M->n, M->row_ptr, M->col, static_cast<const double*>(M->val), du,
                                          f_old, f_int, f_ext, half_dt, con_mask, res, partial);
  ::tfg::note_launch();
  k_cn_sum<<<1, 1024, 0, st>>>(partial, (int)g, sumsq);
  ::tfg::note_launch();
  return check_cuda("fem_heat_cn_residual");
}

}  // extern "C"
