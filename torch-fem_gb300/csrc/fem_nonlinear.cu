// Nonlinear material points fused with element integration:
//
//   Neo-Hookean, finite strain (Hyperelastic3D with
//     psi = mu/2 (tr C - 3) - mu ln J + lambda/2 (ln J)^2,
//     src/torchfem/materials/hyperelasticity.py:66-127 with the psi of
//     benchmarks/hyperelasticity.py:24-30, nlgeom=True in base.py:1050-1076)
//   J2 plasticity, plane strain, linear hardening sigma_f(q) = sigma_y + H q
//     (IsotropicPlasticityPlaneStrain, materials/plasticity.py:430-590)
//
// Each kernel is one thread per element looping over its integration points:
// it forms the increment gradient H from the nodal field, runs the material
// update, accumulates the element forces f_e = sum w detJ t B^T P, and writes
// the optional per-point outputs (stress, state, tangent, F).  The vjp
// kernels recompute the point update from the saved inputs (the increment's
// checkpoint) and pull cotangents back through it by hand.
#include "fem_common.cuh"

namespace tfg {

int etype_info(int etype, int* ne, int* d, int* nip);

template <int NE, int D>
__device__ __forceinline__ void load_field_nl(const double* __restrict__ v, const int32_t* __restrict__ conn,
                                              const uint8_t* __restrict__ con_mask,
                                              const double* __restrict__ con_values, int con_mode,
                                              double (&ve)[NE][D]) {
#pragma unroll
  for (int a = 0; a < NE; ++a) {
    const int64_t nd = conn[a];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const int64_t dof = nd * D + c;
      double x = v ? v[dof] : 0.0;
      if (con_mode != 0 && con_mask[dof]) x = (con_mode == 1) ? con_values[dof] : 0.0;
      ve[a][c] = x;
    }
  }
}

__device__ __forceinline__ double det3(const double (&F)[3][3]) {
  return F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) -
         F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
         F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
}

__device__ __forceinline__ void inv3(const double (&F)[3][3], double J, double (&Fi)[3][3]) {
  const double r = 1.0 / J;
  Fi[0][0] = (F[1][1] * F[2][2] - F[1][2] * F[2][1]) * r;
  Fi[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * r;
  Fi[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * r;
  Fi[1][0] = (F[1][2] * F[2][0] - F[1][0] * F[2][2]) * r;
  Fi[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * r;
  Fi[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * r;
  Fi[2][0] = (F[1][0] * F[2][1] - F[1][1] * F[2][0]) * r;
  Fi[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * r;
  Fi[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * r;
}

// ------------------------------------------------------------ Neo-Hookean ---
// P = mu F + (lambda ln J - mu) F^-T
// A_iJkL = mu d_ik d_JL + lambda Fi_Ji Fi_Lk + (mu - lambda ln J) Fi_Jk Fi_Li
template <int NE, int NIP>
__global__ void __launch_bounds__(128)
k_hyper(const double* __restrict__ bt, const double* __restrict__ detj,
        const double* __restrict__ weights, const int32_t* __restrict__ elements, int64_t n_elem,
        const double* __restrict__ params, const double* __restrict__ v,
        const uint8_t* __restrict__ con_mask, const double* __restrict__ con_values, int con_mode,
        const double* __restrict__ F_prev, double* __restrict__ fe, double* __restrict__ P_out,
        double* __restrict__ tangent, double* __restrict__ flux, double* __restrict__ F_out,
        int32_t* status) {
  constexpr int D = 3, ND = NE * D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  double ve[NE][D];
  load_field_nl<NE, D>(v, elements + e * NE, con_mask, con_values, con_mode, ve);
  const double mu = params[e * 2 + 0], lam = params[e * 2 + 1];
  double f[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) f[a][c] = 0.0;
  bool ok = true;
  for (int ip = 0; ip < NIP; ++ip) {
    const int64_t pe = (int64_t)ip * n_elem + e;
    const double* g = bt + pe * ND;
    double F[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double s = F_prev[pe * 9 + c * 3 + j];
#pragma unroll
        for (int a = 0; a < NE; ++a) s += ve[a][c] * g[a * D + j];
        F[c][j] = s;
      }
    const double J = det3(F);
    ok = ok && (J > 0.0);
    double Fi[3][3];
    inv3(F, J, Fi);
    const double lnJ = log(J);
    const double cm = lam * lnJ - mu;
    double P[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = mu * F[i][j] + cm * Fi[j][i];
    if (P_out) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) P_out[pe * 9 + i * 3 + j] = P[i][j];
    }
    if (F_out) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F_out[pe * 9 + i * 3 + j] = F[i][j];
    }
    if (flux) {  // (F P) / J, base.py:1072-1074
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < 3; ++k) s += F[i][k] * P[k][j];
          flux[pe * 9 + i * 3 + j] = s / J;
        }
    }
    if (tangent) {
      const double c2 = mu - lam * lnJ;
      double* A = tangent + pe * 81;
      for (int i = 0; i < 3; ++i)
        for (int J2 = 0; J2 < 3; ++J2)
          for (int k = 0; k < 3; ++k)
            for (int L = 0; L < 3; ++L)
              A[((i * 3 + J2) * 3 + k) * 3 + L] = (i == k && J2 == L ? mu : 0.0) + lam * Fi[J2][i] * Fi[L][k] +
                                                  c2 * Fi[J2][k] * Fi[L][i];
    }
    const double s = weights[ip] * detj[pe];
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) acc += g[a * D + j] * P[c][j];
        f[a][c] += s * acc;
      }
  }
  double* out = fe + e * ND;
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) {
      out[a * D + c] = f[a][c];
      ok = ok && isfinite(f[a][c]);
    }
  if (!ok) flag_status(status, kStatNonFinite);
}

template <int NE, int NIP>
__global__ void __launch_bounds__(128)
k_hyper_vjp(const double* __restrict__ bt, const double* __restrict__ detj,
            const double* __restrict__ weights, const int32_t* __restrict__ elements, int64_t n_elem,
            const double* __restrict__ params, const double* __restrict__ v,
            const uint8_t* __restrict__ con_mask, const double* __restrict__ con_values, int con_mode,
            const double* __restrict__ F_prev, const double* __restrict__ g_nodal,
            const double* __restrict__ gflux, const double* __restrict__ gF, double* __restrict__ gFprev,
            double* __restrict__ gparams, double* __restrict__ gve) {
  constexpr int D = 3, ND = NE * D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int32_t* conn = elements + e * NE;
  double ve[NE][D], ge[NE][D];
  load_field_nl<NE, D>(v, conn, con_mask, con_values, con_mode, ve);
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) ge[a][c] = g_nodal ? g_nodal[(int64_t)conn[a] * D + c] : 0.0;
  const double mu = params[e * 2 + 0], lam = params[e * 2 + 1];
  double gv[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) gv[a][c] = 0.0;
  double gmu = 0.0, glam = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const int64_t pe = (int64_t)ip * n_elem + e;
    const double* g = bt + pe * ND;
    double F[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double s = F_prev[pe * 9 + c * 3 + j];
#pragma unroll
        for (int a = 0; a < NE; ++a) s += ve[a][c] * g[a * D + j];
        F[c][j] = s;
      }
    const double J = det3(F);
    double Fi[3][3];
    inv3(F, J, Fi);
    const double lnJ = log(J);
    const double cm = lam * lnJ - mu;
    double P[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = mu * F[i][j] + cm * Fi[j][i];
    const double s = weights[ip] * detj[pe];
    // cotangent of P from the forces
    double Pb[3][3], Fb[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
#pragma unroll
        for (int a = 0; a < NE; ++a) acc += ge[a][c] * g[a * D + j];
        Pb[c][j] = s * acc;
        Fb[c][j] = gF ? gF[pe * 9 + c * 3 + j] : 0.0;
      }
    if (gflux) {  // flux = F P / J
      const double* G = gflux + pe * 9;
      double flx[3][3], GF = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double t = 0.0;
#pragma unroll
          for (int k = 0; k < 3; ++k) t += F[i][k] * P[k][j];
          flx[i][j] = t / J;
          GF += G[i * 3 + j] * flx[i][j];
        }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          double t1 = 0.0, t2 = 0.0;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            t1 += G[i * 3 + j] * P[k][j];  // (G P^T)_ik
            t2 += F[j][i] * G[j * 3 + k];  // (F^T G)_ik
          }
          Fb[i][k] += t1 / J - GF * Fi[k][i];
          Pb[i][k] += t2 / J;
        }
    }
    // A : Pb = mu Pb + lam tr(Fi Pb) Fi^T + (mu - lam lnJ) (Fi Pb Fi)^T
    double T = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) T += Fi[i][j] * Pb[j][i];
    double M[3][3];  // Fi Pb Fi
#pragma unroll
    for (int L = 0; L < 3; ++L)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double t = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) t += Fi[L][i] * Pb[i][j] * Fi[j][k];
        M[L][k] = t;
      }
    const double c2 = mu - lam * lnJ;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int L = 0; L < 3; ++L) Fb[k][L] += mu * Pb[k][L] + lam * T * Fi[L][k] + c2 * M[L][k];
    // parameters: dP/dmu = F - F^-T, dP/dlam = lnJ F^-T
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        gmu += Pb[i][j] * (F[i][j] - Fi[j][i]);
        glam += Pb[i][j] * lnJ * Fi[j][i];
      }
    if (gFprev) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) gFprev[pe * 9 + i * 3 + j] = Fb[i][j];
    }
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) acc += g[a * D + j] * Fb[c][j];
        gv[a][c] += acc;
      }
  }
  if (gparams) {
    gparams[e * 2 + 0] = gmu;
    gparams[e * 2 + 1] = glam;
  }
  if (gve) {
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) gve[e * ND + a * D + c] = gv[a][c];
  }
}

// ------------------------------------------------ J2 plasticity, plane strain
// params [n_elem][4] = (E, nu, sigma_y, H); state [.., 2] = (q, eps_z^p).
struct J2Point {
  double s3[3][3];  // trial stress (3D, zz from plane strain)
  double dev[3][3];
  double nrm;
  double dG;        // plastic multiplier (0 if elastic)
  double q_new;
  bool plastic;
};

__device__ __forceinline__ void j2_update(double lam, double G, double E, double nu, double sy, double Hh,
                                          const double (&eps)[2][2], const double* sp, double q, double ez,
                                          double tol, int max_iter, J2Point& o) {
  double s2[2][2];
  const double tr = eps[0][0] + eps[1][1];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
      s2[i][j] = (sp ? sp[i * 2 + j] : 0.0) + G * (eps[i][j] + eps[j][i]) + (i == j ? lam * tr : 0.0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.s3[i][j] = 0.0;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) o.s3[i][j] = s2[i][j];
  o.s3[2][2] = nu * (s2[0][0] + s2[1][1]) - E * ez;
  const double t3 = (o.s3[0][0] + o.s3[1][1] + o.s3[2][2]) / 3.0;
  double n2 = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      o.dev[i][j] = o.s3[i][j] - (i == j ? t3 : 0.0);
      n2 += o.dev[i][j] * o.dev[i][j];
    }
  o.nrm = sqrt(n2);
  const double c = sqrt(2.0 / 3.0);
  const double f = o.nrm - c * (sy + Hh * q);
  o.plastic = f > 0.0;
  o.dG = 0.0;
  o.q_new = q;
  if (o.plastic) {
    // local Newton of plasticity.py:548-560 (exact after one step for linear hardening)
    double dG = 0.0, qc = q;
    for (int it = 0; it < max_iter; ++it) {
      const double res = o.nrm - 2.0 * G * dG - c * (sy + Hh * qc);
      const double dd = res / (2.0 * G + 2.0 / 3.0 * Hh);
      dG += dd;
      qc += c * dd;
      if (fabs(res) < tol) break;
    }
    o.dG = dG;
    o.q_new = qc;
  }
}

template <int NE, int NIP>
__global__ void __launch_bounds__(128)
k_plastic(const double* __restrict__ bt, const double* __restrict__ detj,
          const double* __restrict__ weights, const double* __restrict__ thickness,
          const int32_t* __restrict__ elements, int64_t n_elem, const double* __restrict__ params,
          double tol, int max_iter, const double* __restrict__ v, const uint8_t* __restrict__ con_mask,
          const double* __restrict__ con_values, int con_mode, const double* __restrict__ sigma_prev,
          const double* __restrict__ state_prev, const double* __restrict__ de0, double* __restrict__ fe,
          double* __restrict__ sigma_out, double* __restrict__ state_out, double* __restrict__ tangent,
          double* __restrict__ hgrad, int32_t* status) {
  constexpr int D = 2, ND = NE * D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  double ve[NE][D];
  load_field_nl<NE, D>(v, elements + e * NE, con_mask, con_values, con_mode, ve);
  const double E = params[e * 4 + 0], nu = params[e * 4 + 1], sy = params[e * 4 + 2], Hh = params[e * 4 + 3];
  const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), G = E / (2.0 * (1.0 + nu));
  const double th = thickness ? thickness[e] : 1.0;
  double f[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) f[a][c] = 0.0;
  bool ok = true;
  for (int ip = 0; ip < NIP; ++ip) {
    const int64_t pe = (int64_t)ip * n_elem + e;
    const double* g = bt + pe * ND;
    double H[2][2];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < NE; ++a) s += ve[a][c] * g[a * D + j];
        H[c][j] = s;
      }
    if (hgrad) {
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) hgrad[pe * 4 + i * 2 + j] = H[i][j];
    }
    double eps[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) eps[i][j] = 0.5 * (H[i][j] + H[j][i]) - (de0 ? de0[e * 4 + i * 2 + j] : 0.0);
    const double q = state_prev ? state_prev[pe * 2 + 0] : 0.0;
    const double ez = state_prev ? state_prev[pe * 2 + 1] : 0.0;
    J2Point o;
    j2_update(lam, G, E, nu, sy, Hh, eps, sigma_prev ? sigma_prev + pe * 4 : nullptr, q, ez, tol, max_iter, o);
    double sig[2][2];
    double nn[3][3];
    if (o.plastic) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) nn[i][j] = o.dev[i][j] / o.nrm;
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) sig[i][j] = o.s3[i][j] - 2.0 * G * o.dG * nn[i][j];
    } else {
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) sig[i][j] = o.s3[i][j];
    }
    if (sigma_out) {
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) sigma_out[pe * 4 + i * 2 + j] = sig[i][j];
    }
    if (state_out) {
      state_out[pe * 2 + 0] = o.q_new;
      state_out[pe * 2 + 1] = o.plastic ? ez + o.dG * nn[2][2] : ez;
    }
    if (tangent) {  // plasticity.py:577-588
      double T[2][2][2][2];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          for (int k = 0; k < 2; ++k)
            for (int l = 0; l < 2; ++l) T[i][j][k][l] = 0.0;
      T[0][0][0][0] = 2.0 * G + lam;
      T[1][1][1][1] = 2.0 * G + lam;
      T[0][0][1][1] = lam;
      T[1][1][0][0] = lam;
      T[0][1][0][1] = G;
      T[0][1][1][0] = G;
      T[1][0][0][1] = G;
      T[1][0][1][0] = G;
      if (o.plastic) {
        const double Ac = 2.0 * G / (1.0 + Hh / (3.0 * G));
        const double Bc = 4.0 * G * G * o.dG / o.nrm;
        const double n0n1 = nn[0][0] * nn[1][1];
        T[0][0][0][0] += -Ac * nn[0][0] * nn[0][0] - Bc * (2.0 / 3.0 - nn[0][0] * nn[0][0]);
        T[1][1][1][1] += -Ac * nn[1][1] * nn[1][1] - Bc * (2.0 / 3.0 - nn[1][1] * nn[1][1]);
        T[0][0][1][1] += -Ac * n0n1 - Bc * (-1.0 / 3.0 - n0n1);
        T[1][1][0][0] += -Ac * n0n1 - Bc * (-1.0 / 3.0 - n0n1);
        T[0][1][0][1] += -Ac * nn[0][1] * nn[0][1] - Bc * (0.5 - nn[0][1] * nn[0][1]);
        T[0][1][1][0] += -Ac * nn[0][1] * nn[0][1] - Bc * (0.5 - nn[1][0] * nn[1][0]);
        T[1][0][0][1] += -Ac * nn[1][0] * nn[1][0] - Bc * (0.5 - nn[0][1] * nn[0][1]);
        T[1][0][1][0] += -Ac * nn[1][0] * nn[1][0] - Bc * (0.5 - nn[1][0] * nn[1][0]);
      }
      double* Tp = tangent + pe * 16;
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          for (int k = 0; k < 2; ++k)
            for (int l = 0; l < 2; ++l) Tp[((i * 2 + j) * 2 + k) * 2 + l] = T[i][j][k][l];
    }
    const double s = weights[ip] * detj[pe] * th;
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) acc += g[a * D + j] * sig[c][j];
        f[a][c] += s * acc;
      }
  }
  double* out = fe + e * ND;
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) {
      out[a * D + c] = f[a][c];
      ok = ok && isfinite(f[a][c]);
    }
  if (!ok) flag_status(status, kStatNonFinite);
}

// Reverse of k_plastic at the saved inputs (one increment's checkpoint).
template <int NE, int NIP>
__global__ void __launch_bounds__(128)
k_plastic_vjp(const double* __restrict__ bt, const double* __restrict__ detj,
              const double* __restrict__ weights, const double* __restrict__ thickness,
              const int32_t* __restrict__ elements, int64_t n_elem, const double* __restrict__ params,
              double tol, int max_iter, const double* __restrict__ v,
              const uint8_t* __restrict__ con_mask, const double* __restrict__ con_values, int con_mode,
              const double* __restrict__ sigma_prev, const double* __restrict__ state_prev,
              const double* __restrict__ de0, const double* __restrict__ g_nodal,
              const double* __restrict__ gsig_out, const double* __restrict__ gstate_out,
              const double* __restrict__ gh, double* __restrict__ gsig_prev,
              double* __restrict__ gstate_prev, double* __restrict__ gthick, double* __restrict__ gve) {
  constexpr int D = 2, ND = NE * D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int32_t* conn = elements + e * NE;
  double ve[NE][D], ge[NE][D];
  load_field_nl<NE, D>(v, conn, con_mask, con_values, con_mode, ve);
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) ge[a][c] = g_nodal ? g_nodal[(int64_t)conn[a] * D + c] : 0.0;
  const double E = params[e * 4 + 0], nu = params[e * 4 + 1], sy = params[e * 4 + 2], Hh = params[e * 4 + 3];
  const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), G = E / (2.0 * (1.0 + nu));
  const double th = thickness ? thickness[e] : 1.0;
  const double cc = sqrt(2.0 / 3.0);
  double gv[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) gv[a][c] = 0.0;
  double gt = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const int64_t pe = (int64_t)ip * n_elem + e;
    const double* g = bt + pe * ND;
    double H[2][2], gradg[2][2];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        double s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int a = 0; a < NE; ++a) {
          s1 += ve[a][c] * g[a * D + j];
          s2 += ge[a][c] * g[a * D + j];
        }
        H[c][j] = s1;
        gradg[c][j] = s2;
      }
    double eps[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) eps[i][j] = 0.5 * (H[i][j] + H[j][i]) - (de0 ? de0[e * 4 + i * 2 + j] : 0.0);
    const double q = state_prev ? state_prev[pe * 2 + 0] : 0.0;
    const double ez = state_prev ? state_prev[pe * 2 + 1] : 0.0;
    J2Point o;
    j2_update(lam, G, E, nu, sy, Hh, eps, sigma_prev ? sigma_prev + pe * 4 : nullptr, q, ez, tol, max_iter, o);
    const double wd = weights[ip] * detj[pe];
    const double s = wd * th;
    double nn[3][3];
    double sig[2][2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) nn[i][j] = o.plastic ? o.dev[i][j] / o.nrm : 0.0;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) sig[i][j] = o.s3[i][j] - (o.plastic ? 2.0 * G * o.dG * nn[i][j] : 0.0);
    if (gthick) {
      double acc = 0.0;
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc += gradg[i][j] * sig[i][j];
      gt += wd * acc;
    }
    // cotangents of the point outputs
    double sb[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) sb[i][j] = s * gradg[i][j] + (gsig_out ? gsig_out[pe * 4 + i * 2 + j] : 0.0);
    const double qb = gstate_out ? gstate_out[pe * 2 + 0] : 0.0;
    const double ezb = gstate_out ? gstate_out[pe * 2 + 1] : 0.0;
    double S3b[3][3];  // cotangent of the 3D trial stress
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S3b[i][j] = (i < 2 && j < 2) ? sb[i][j] : 0.0;
    double q_prev_b = qb, ez_prev_b = ezb;
    if (o.plastic) {
      const double a = o.dG;
      // a-bar from sigma_new = s3 - 2G a n (2x2), q_new = q + c a, ez_new = ez + a n_zz
      double ab = qb * cc + ezb * nn[2][2];
      double nb[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) nb[i][j] = 0.0;
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          ab += sb[i][j] * (-2.0 * G * nn[i][j]);
          nb[i][j] = -2.0 * G * a * sb[i][j];
        }
      nb[2][2] += ezb * a;
      // a = f / (2G + 2H/3), f = nrm - c (sy + H q)
      const double fb = ab / (2.0 * G + 2.0 / 3.0 * Hh);
      double nrmb = fb;
      q_prev_b += -cc * Hh * fb;
      // n = dev / nrm
      double nbn = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) nbn += nb[i][j] * nn[i][j];
      nrmb += -nbn / o.nrm;  // n = dev / nrm: d n / d nrm = -n / nrm
      double devb[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) devb[i][j] = nb[i][j] / o.nrm + nrmb * nn[i][j];
      // dev = s3 - tr/3 I: deviatoric projection is self-adjoint
      const double trb = (devb[0][0] + devb[1][1] + devb[2][2]) / 3.0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S3b[i][j] += devb[i][j] - (i == j ? trb : 0.0);
    }
    // s3: 2x2 block s2, s3_zz = nu (s2_00 + s2_11) - E ez
    double s2b[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) s2b[i][j] = S3b[i][j] + (i == j ? nu * S3b[2][2] : 0.0);
    ez_prev_b += -E * S3b[2][2];
    if (gsig_prev) {
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) gsig_prev[pe * 4 + i * 2 + j] = s2b[i][j];
    }
    if (gstate_prev) {
      gstate_prev[pe * 2 + 0] = q_prev_b;
      gstate_prev[pe * 2 + 1] = ez_prev_b;
    }
    // s2 = sigma_prev + C:eps (C isotropic, major symmetric) -> eps-bar = C:s2b
    double trs = s2b[0][0] + s2b[1][1];
    double Hb[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const double eb_ij = G * (s2b[i][j] + s2b[j][i]) + (i == j ? lam * trs : 0.0);
        const double eb_ji = G * (s2b[j][i] + s2b[i][j]) + (i == j ? lam * trs : 0.0);
        Hb[i][j] = 0.5 * (eb_ij + eb_ji) + (gh ? gh[pe * 4 + i * 2 + j] : 0.0);
      }
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) acc += g[a * D + j] * Hb[c][j];
        gv[a][c] += acc;
      }
  }
  if (gthick) gthick[e] = gt;
  if (gve) {
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) gve[e * ND + a * D + c] = gv[a][c];
  }
}

}  // namespace tfg

using namespace tfg;

#define TFG_NL3_DISPATCH(etype)                                   \
  switch (etype) {                                                \
    case FEM_HEXA1: { constexpr int NE = 8, NIP = 8; TFG_BODY; } break;   \
    case FEM_TETRA2: { constexpr int NE = 10, NIP = 4; TFG_BODY; } break; \
    case FEM_TETRA1: { constexpr int NE = 4, NIP = 1; TFG_BODY; } break;  \
    default:                                                      \
      set_last_error("element type %d has no 3D finite-strain kernel", etype); \
      return FEM_INVALID;                                         \
  }

#define TFG_NL2_DISPATCH(etype)                                   \
  switch (etype) {                                                \
    case FEM_QUAD1: { constexpr int NE = 4, NIP = 4; TFG_BODY; } break;  \
    case FEM_TRIA1: { constexpr int NE = 3, NIP = 1; TFG_BODY; } break;  \
    case FEM_QUAD2: { constexpr int NE = 8, NIP = 4; TFG_BODY; } break;  \
    case FEM_TRIA2: { constexpr int NE = 6, NIP = 3; TFG_BODY; } break;  \
    default:                                                      \
      set_last_error("element type %d has no plane-strain plasticity kernel", etype); \
      return FEM_INVALID;                                         \
  }

extern "C" {

int fem_hyper_force(const fem_mesh* m, const double* params, const double* v, const uint8_t* con_mask,
                    const double* con_values, int con_mode, const double* F_prev, double* fe, double* P_out,
                    double* tangent, double* flux, double* F_out, int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
#define TFG_BODY                                                                                   \
  k_hyper<NE, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                      \
      m->bt, m->detj, m->weights, m->elements, m->n_elem, params, v, con_mask, con_values, con_mode, \
      F_prev, fe, P_out, tangent, flux, F_out, status);
  TFG_NL3_DISPATCH(m->etype)
#undef TFG_BODY
  ::tfg::note_launch();
  return check_cuda("fem_hyper_force");
}

int fem_hyper_vjp(const fem_mesh* m, const double* params, const double* v, const uint8_t* con_mask,
                  const double* con_values, int con_mode, const double* F_prev, const double* g,
                  const double* gflux, const double* gF, double* gFprev, double* gparams, double* gve,
                  void* stream) {
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
#define TFG_BODY                                                                                    \
  k_hyper_vjp<NE, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                   \
      m->bt, m->detj, m->weights, m->elements, m->n_elem, params, v, con_mask, con_values, con_mode, \
      F_prev, g, gflux, gF, gFprev, gparams, gve);
  TFG_NL3_DISPATCH(m->etype)
#undef TFG_BODY
  ::tfg::note_launch();
  return check_cuda("fem_hyper_vjp");
}

int fem_plastic_force(const fem_mesh* m, const double* params, double tol, int max_iter, const double* v,
                      const uint8_t* con_mask, const double* con_values, int con_mode,
                      const double* sigma_prev, const double* state_prev, const double* de0, double* fe,
                      double* sigma_out, double* state_out, double* tangent, double* hgrad,
                      int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
#define TFG_BODY                                                                                    \
  k_plastic<NE, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                     \
      m->bt, m->detj, m->weights, m->thickness, m->elements, m->n_elem, params, tol, max_iter, v,    \
      con_mask, con_values, con_mode, sigma_prev, state_prev, de0, fe, sigma_out, state_out, tangent, \
      hgrad, status);
  TFG_NL2_DISPATCH(m->etype)
#undef TFG_BODY
  ::tfg::note_launch();
  return check_cuda("fem_plastic_force");
}

int fem_plastic_vjp(const fem_mesh* m, const double* params, double tol, int max_iter, const double* v,
                    const uint8_t* con_mask, const double* con_values, int con_mode,
                    const double* sigma_prev, const double* state_prev, const double* de0, const double* g,
                    const double* gsig_out, const double* gstate_out, const double* ghgrad,
                    double* gsig_prev, double* gstate_prev, double* gthick, double* gve, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
#define TFG_BODY                                                                                     \
  k_plastic_vjp<NE, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                  \
      m->bt, m->detj, m->weights, m->thickness, m->elements, m->n_elem, params, tol, max_iter, v,     \
      con_mask, con_values, con_mode, sigma_prev, state_prev, de0, g, gsig_out, gstate_out, ghgrad,   \
      gsig_prev, gstate_prev, gthick, gve);
  TFG_NL2_DISPATCH(m->etype)
#undef TFG_BODY
  ::tfg::note_launch();
  return check_cuda("fem_plastic_vjp");
}

}  // extern "C"
