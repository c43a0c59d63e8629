/*
 * torchfem_gb300.h — C ABI of the GB300 forward + adjoint finite-element path.
 *
 * The library replaces the compute underneath torch-fem's `FEM.solve`
 * (src/torchfem/base.py:597-923): sparsity precompute, Gauss-point element
 * integration, element-to-CSR assembly with Dirichlet condensation, the
 * linear solve behind `sparse_solve` (src/torchfem/sparse.py:271-347) and the
 * adjoint pieces behind `NewtonRaphsonAdjoint.backward`
 * (src/torchfem/sparse.py:641-724).  torch-fem itself is pure Python and has
 * no FFI; each entry point below cites the Python function whose arithmetic it
 * takes over, which is the seam a binding (ctypes, cffi, pybind) attaches to.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers into caller-owned memory unless a
 *    comment says "host".  The library never allocates device memory; entry
 *    points that need scratch take (ws, ws_bytes) sized by the matching
 *    *_workspace_bytes query.
 *  - `stream` is a cudaStream_t passed as void*; all work is ordered on it.
 *    Entry points that return a size to the host synchronise that stream.
 *  - Index types: node ids, column indices and element-contributor codes are
 *    int32; row pointers and slot maps are int64.
 *  - `status` (nullable) is a device int32 word into which kernels OR
 *    (1 << FEM_*) bits for device-detected conditions.
 *  - Degree-of-freedom numbering is node-major, dof = node * dim + component
 *    (src/torchfem/base.py:73-76).
 */
#ifndef TORCHFEM_GB300_H
#define TORCHFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FEM_ABI_VERSION 1

/* Return codes.  The Python host maps them to the reference's exceptions:
 * FEM_NOT_CONVERGED / FEM_NONFINITE / FEM_BREAKDOWN -> RuntimeError
 * (src/torchfem/sparse.py:412-421, :500-512, :622-623), FEM_BAD_JACOBIAN ->
 * ValueError (src/torchfem/base.py:311-312), FEM_INVALID -> ValueError. */
enum {
  FEM_OK = 0,
  FEM_NOT_CONVERGED = 1,
  FEM_NONFINITE = 2,
  FEM_BAD_JACOBIAN = 3,
  FEM_BOUNDS = 4,
  FEM_INVALID = 5,
  FEM_CUDA_ERROR = 6,
  FEM_BREAKDOWN = 7
};

/* Element types (src/torchfem/elements.py).  Shape-function gradient tables
 * and weights are supplied by the caller, so the library does not fix the
 * quadrature; it only fixes (nodes, dim, integration points). */
enum {
  FEM_QUAD1 = 1,  /* 4 nodes, 2D, 4 points   (elements.py:491-567)  */
  FEM_HEXA1 = 2,  /* 8 nodes, 3D, 8 points   (elements.py:936-1075) */
  FEM_TETRA2 = 3, /* 10 nodes, 3D, 4 points  (elements.py:793-933)  */
  FEM_TETRA1 = 4, /* 4 nodes, 3D, 1 point    (elements.py:727-790)  */
  FEM_TRIA1 = 5,  /* 3 nodes, 2D, 1 point    (elements.py:309-382)  */
  FEM_QUAD2 = 6,  /* 8 nodes, 2D, 4 points   (elements.py:570-724)  */
  FEM_TRIA2 = 7,  /* 6 nodes, 2D, 3 points   (elements.py:385-488)  */
  FEM_SHELL3 = 8, /* Tria1 flat-facet shell: 3 nodes, 6 DOF per node (shell.py);
                     used by fem_gather_nodal, the shell kernels take fem_shell */
  FEM_HEXA2 = 9   /* 20 nodes, 3D, 8 points  (elements.py:1078-1406) */
};

/* Material data layouts consumed by the element kernels. */
enum {
  FEM_MAT_ISO = 1,        /* [n_elem][2] = (lambda, G): C = lambda I(x)I + G (I4 sym sum).
                             Covers IsotropicElasticity3D / PlaneStrain and, with effective
                             constants, PlaneStress (materials/elasticity.py:44-241). */
  FEM_MAT_GENERAL = 2,    /* [n_elem][dim^4] full tangent C_iJkL per element. */
  FEM_MAT_TANGENT_IP = 3, /* [nip][n_elem][dim^4] tangent per integration point. */
  FEM_MAT_CONDUCTIVITY = 16 /* [n_elem][dim][dim] conductivity (heat conduction, one DOF
                               per node): fem_element_stiffness / _force / _vjp forward
                               this kind to fem_heat_*, which take the array itself. */
};

enum { FEM_F64 = 0, FEM_F32 = 1 };
enum { FEM_FMT_CSR_F64 = 1, FEM_FMT_SELL_F32 = 2 };

/* Last error message of the calling thread (host string). */
const char* fem_last_error(void);
int fem_abi_version(void);
/* Number of kernels the library has launched in this process (host counter). */
int64_t fem_launch_count(void);

/* ------------------------------------------------------------------------ */
/* Sparsity pattern: FEM.__init__ (src/torchfem/base.py:72-122).            */
/* The reference builds packed 64-bit (row, col) keys, `torch.unique`s them  */
/* and `searchsorted`s every element entry.  Here the pattern is derived     */
/* from the node graph: the DOF pattern is the node adjacency with a dense   */
/* dim x dim block per node pair, plus the diagonal of nodes that belong to  */
/* no element — the same set the reference's keys produce.                   */
/* ------------------------------------------------------------------------ */

size_t fem_pattern_workspace_bytes(int64_t n_nod, int64_t n_elem, int n_e);

/* Node->element incidence (inc: codes e*n_e + local node, ascending per
 * node) and node-neighbour counts scanned into nbr_ptr [n_nod+1].  Writes the
 * number of node-pair blocks to *n_blocks (host). */
int fem_pattern_graph_count(const int32_t* elements, int64_t n_elem, int n_e, int64_t n_nod,
                            int64_t* inc_ptr, int32_t* inc, int64_t* nbr_ptr,
                            int64_t* n_blocks, void* ws, size_t ws_bytes, int32_t* status,
                            void* stream);

/* Sorted node neighbour lists nbr [n_blocks] (each node lists itself). */
int fem_pattern_graph_fill(const int32_t* elements, int64_t n_elem, int n_e, int64_t n_nod,
                           const int64_t* inc_ptr, const int32_t* inc, const int64_t* nbr_ptr,
                           int32_t* nbr, int32_t* status, void* stream);

/* Scalar CSR row pointers [n_dofs+1] of the reference pattern; *nnz (host). */
int fem_pattern_csr_rows(const int64_t* nbr_ptr, int64_t n_nod, int dof_per_node,
                         const int64_t* inc_ptr, int64_t* row_ptr, int64_t* nnz, void* ws,
                         size_t ws_bytes, void* stream);

/* Column indices [nnz] (== glob_idx[1], base.py:112-117) and the slot of
 * each diagonal entry [n_dofs] (== diag_map, base.py:106-108). */
int fem_pattern_csr_cols(const int64_t* nbr_ptr, const int32_t* nbr, int64_t n_nod,
                         int dof_per_node, const int64_t* inc_ptr, const int64_t* row_ptr,
                         int32_t* col, int64_t* diag_map, void* stream);

/* Slot of every element-matrix entry, row-major over (e, p, q) — the
 * reference's k_map (base.py:93-104) — for parity checks and for callers that
 * assemble with it. */
int fem_pattern_kmap(const int32_t* elements, int64_t n_elem, int n_e, int dof_per_node,
                     const int64_t* nbr_ptr, const int32_t* nbr, const int64_t* row_ptr,
                     int64_t* k_map, int32_t* status, void* stream);

/* Block-level contributor lists used by the atomic-free assembly: for block b
 * (a node pair), contrib[blk_ptr[b] .. blk_ptr[b+1]) are codes
 * (e*n_e + la)*n_e + lb in ascending element order, which is the order in
 * which CPU index_add_ visits them (base.py:410-411).  blk_row [n_blocks]
 * is the row node of each block, diag_blk [n_nod] the block (a, a). */
int fem_pattern_blocks(const int32_t* elements, int64_t n_elem, int n_e, int64_t n_nod,
                       const int64_t* inc_ptr, const int32_t* inc, const int64_t* nbr_ptr,
                       const int32_t* nbr, int64_t n_blocks, int64_t* blk_ptr,
                       int32_t* contrib, int32_t* blk_row, int64_t* diag_blk, void* ws,
                       size_t ws_bytes, int32_t* status, void* stream);

/* ------------------------------------------------------------------------ */
/* Element integration: eval_shape_functions (base.py:293-314) and           */
/* Mechanics.integrate_material (base.py:982-1092).                          */
/* ------------------------------------------------------------------------ */

typedef struct fem_mesh {
  int etype;               /* FEM_* element type */
  int64_t n_nod;
  int64_t n_elem;
  const double* nodes;     /* [n_nod][dim] */
  const int32_t* elements; /* [n_elem][n_e] */
  const double* weights;   /* [nip] integration weights */
  const double* bt;        /* [nip][n_elem][n_e][dim] dN/dx (fem_geometry output) */
  const double* detj;      /* [nip][n_elem] */
  const int64_t* inc_ptr;  /* [n_nod+1] node->element incidence */
  const int32_t* inc;      /* [n_elem*n_e] */
  const double* thickness; /* [n_elem] planar thickness, NULL for solids */
  int dof_per_node;        /* DOFs per node of the field (0: the element's dimension; 1 for
                              heat conduction) */
} fem_mesh;

typedef struct fem_material {
  int kind;                /* FEM_MAT_* */
  const double* data;
} fem_material;

/* Jacobian, its determinant and the physical shape-function gradients at
 * every integration point (base.py:306-313).  dndxi is [nip][dim][n_e].
 * detJ <= 0 flags FEM_BAD_JACOBIAN in *status. */
int fem_geometry(const fem_mesh* mesh, const double* dndxi, double* bt, double* detj,
                 int32_t* status, void* stream);

/* Element stiffness Ke = sum_ip w detJ t B^T C B (base.py:1085-1090,
 * solid.py:52-54, planar.py:86-88), stored [n_elem][n_e*dim][n_e*dim] in
 * out_dtype (FEM_F64 or FEM_F32). */
int fem_element_stiffness(const fem_mesh* mesh, const fem_material* mat, int out_dtype,
                          void* ke, int32_t* status, void* stream);

/* The same FP64 element matrices for an isotropic material (FEM_MAT_ISO),
 * regrouped as K_ab = lambda M + G M^T + G tr(M) I with the moments
 * M = sum_ip w detJ t g_a g_b^T, one thread per node pair a <= b: the FP64
 * element matrices of the mixed solvers' FP64 matrix copy
 * (fem_assemble_sell_pair).  Equal to fem_element_stiffness(FEM_F64) up to
 * summation order; no counterpart in the reference. */
int fem_element_stiffness_iso64(const fem_mesh* mesh, const fem_material* mat, double* ke,
                                int32_t* status, void* stream);

/* Element internal forces f_e = sum_ip w detJ t B^T sigma with the linear
 * stress update sigma = sigma_prev + C:(sym grad v - de0) (base.py:1050-1083,
 * elasticity.py:119-127).  con_mode: 0 use v as is, 1 replace v at
 * constrained DOFs by con_values (du_bc, base.py:710-711), 2 zero v there.
 * sigma_prev [nip][n_elem][dim][dim] and de0 [n_elem][dim][dim] are
 * nullable.  fe [n_elem][n_e][dim]; flux [nip][n_elem][dim][dim] and the
 * increment gradient hgrad = H_inc [nip][n_elem][dim][dim] (base.py:1052)
 * are nullable outputs. */
int fem_element_force(const fem_mesh* mesh, const fem_material* mat, const double* v,
                      const uint8_t* con_mask, const double* con_values, int con_mode,
                      const double* sigma_prev, const double* de0, double* fe, double* flux,
                      double* hgrad, int32_t* status, void* stream);

/* Deterministic nodal assembly of element vectors (assemble_rhs,
 * base.py:428-445): out[dof] = sum over the node's incident elements in
 * ascending order, starting from +0.0 — the serial order of CPU index_add_.
 * If sub != NULL, out = gathered - sub.  con_mode: 0 none, 1 zero at
 * constrained DOFs (res[con] = 0, base.py:738-739), 2 copy con_src there.
 * Optional *sumsq (device, nullable) receives ||out||^2 and then needs a
 * workspace of fem_gather_workspace_bytes(n_nod*dim). */
size_t fem_gather_workspace_bytes(int64_t n);
int fem_gather_nodal(const fem_mesh* mesh, const double* fe, const double* sub,
                     const uint8_t* con_mask, int con_mode, const double* con_src, double* out,
                     double* sumsq, void* ws, size_t ws_bytes, void* stream);

/* Vector-Jacobian product of fem_element_force for the hand-written adjoint
 * (replaces torch.autograd.grad at sparse.py:698-705).  Given the cotangent
 * g of the assembled forces (nodal, [n_nod*dim]), of the flux output
 * (gflux, nullable) and of the hgrad output (ghgrad, nullable), writes the
 * nullable cotangents of: sigma_prev
 * (gsig [nip][n_elem][dim][dim]), material data (gmat, layout of mat->data),
 * thickness (gthick [n_elem]), de0 (gde0 [n_elem][dim][dim]) and of the
 * per-element input field (gve [n_elem][n_e][dim], gather with
 * fem_gather_nodal).  v/con_* as in fem_element_force. */
int fem_element_vjp(const fem_mesh* mesh, const fem_material* mat, const double* v,
                    const uint8_t* con_mask, const double* con_values, int con_mode,
                    const double* sigma_prev, const double* de0, const double* g,
                    const double* gflux, const double* ghgrad, double* gsig, double* gmat,
                    double* gthick, double* gde0, double* gve, int32_t* status, void* stream);

/* ------------------------------------------------------------------------ */
/* Heat conduction: one temperature DOF per node (mesh->dof_per_node = 1).  */
/* ------------------------------------------------------------------------ */
/* kappa [n_elem][dim][dim] is the conductivity tensor of the Fourier law of
 * materials/conductivity.py:80-99 (flux = flux_prev + kappa (grad_inc -
 * de0), tangent kappa).  Point arrays (flux_prev, flux, hgrad, gflux, ...)
 * are [nip][n_elem][dim], the reference's [n_int][n_elem][1][dim]. */

/* Element conductivity matrices k_ab = sum_ip w detJ t B_a . kappa B_b
 * [n_elem][n_e][n_e] in out_dtype: the stiffness part of
 * Heat.integrate_material (base.py:1177-1286) with compute_k
 * (solid.py:52-54, planar.py:86-88); also Heat.k0 (base.py:228-245). */
int fem_heat_stiffness(const fem_mesh* mesh, const double* kappa, int out_dtype, void* ke,
                       int32_t* status, void* stream);

/* Nodal heat fluxes of a temperature increment v [n_nod] (constrained
 * entries replaced per con_mode as in fem_element_force): f_a = sum_ip w
 * detJ t B_a . flux (compute_f, solid.py:56-58, planar.py:90-92), with the
 * updated point fluxes (flux) and the gradient increments (hgrad) as
 * optional outputs (base.py:1236-1262).  de0 [n_elem][dim] may be NULL. */
int fem_heat_force(const fem_mesh* mesh, const double* kappa, const double* v,
                   const uint8_t* con_mask, const double* con_values, int con_mode,
                   const double* flux_prev, const double* de0, double* fe, double* flux,
                   double* hgrad, int32_t* status, void* stream);

/* Vector-Jacobian product of fem_heat_force: cotangents g (assembled heat
 * fluxes [n_nod]), gflux and ghgrad (point outputs) pulled back to flux_prev
 * (gflux_prev), kappa (gkappa [n_elem][dim][dim]), the thickness (gthick),
 * de0 (gde0 [n_elem][dim]) and the element temperatures (gve [n_elem][n_e],
 * gather with fem_gather_nodal).  Every output is nullable. */
int fem_heat_vjp(const fem_mesh* mesh, const double* kappa, const double* v,
                 const uint8_t* con_mask, const double* con_values, int con_mode,
                 const double* flux_prev, const double* de0, const double* g, const double* gflux,
                 const double* ghgrad, double* gflux_prev, double* gkappa, double* gthick,
                 double* gde0, double* gve, void* stream);

/* Element capacity (mass) matrices m_ab = sum_ip w detJ t rho N_a N_b
 * [n_elem][n_e][n_e] of FEM.integrate_mass (base.py:376-396) with compute_m
 * (solid.py:60-62, planar.py:94-96) for one DOF per node; rho [n_elem],
 * nval [nip][n_e] the shape-function values at the integration points. */
int fem_heat_mass(const fem_mesh* mesh, const double* rho, const double* nval, int out_dtype,
                  void* me, int32_t* status, void* stream);

/* Vector-Jacobian product of the capacity matrices: out[e] = sum_ip w detJ
 * (N . a_e)(N . b_e) for nodal vectors a, b [n_nod], i.e. a_e^T m_e b_e /
 * (rho_e t_e).  The caller scales it into d/d rho_e and d/d t_e of a^T M b:
 * the parameter pull-back of the capacity term M du of the Crank-Nicolson
 * residual that the reference's time_integration differentiates by autograd
 * (base.py:376-396 with solid.py:60-62 / planar.py:94-96, base.py:1288-1553). */
int fem_heat_mass_vjp(const fem_mesh* mesh, const double* nval, const double* a, const double* b, double* out,
                      void* stream);


/* ------------------------------------------------------------------------ */
/* Nonlinear material points fused with element integration.                */
/* ------------------------------------------------------------------------ */

/* Neo-Hookean solid at finite strain (Hyperelastic3D with
 * psi = mu/2 (tr C - 3) - mu ln J + lambda/2 (ln J)^2, hyperelasticity.py:66-127,
 * integrated with nlgeom as in base.py:1050-1083).  params [n_elem][2] =
 * (mu, lambda).  Per point F = F_prev + grad(v) (F_prev, F_out
 * [nip][n_elem][3][3]), P = dpsi/dF (P_out), tangent A = d2psi/dF2
 * [nip][n_elem][81], flux = F P / J (base.py:1072-1074); all outputs but fe
 * nullable.  v / con_* as in fem_element_force. */
int fem_hyper_force(const fem_mesh* mesh, const double* params, const double* v,
                    const uint8_t* con_mask, const double* con_values, int con_mode,
                    const double* F_prev, double* fe, double* P_out, double* tangent,
                    double* flux, double* F_out, int32_t* status, void* stream);

/* Vector-Jacobian product of fem_hyper_force: cotangents g (assembled
 * forces), gflux and gF (point outputs) pulled back to F_prev (gFprev),
 * params (gparams [n_elem][2]) and the element field (gve). */
int fem_hyper_vjp(const fem_mesh* mesh, const double* params, const double* v,
                  const uint8_t* con_mask, const double* con_values, int con_mode,
                  const double* F_prev, const double* g, const double* gflux, const double* gF,
                  double* gFprev, double* gparams, double* gve, void* stream);

/* J2 plasticity in plane strain with linear hardening sigma_f = sigma_y + H q
 * (IsotropicPlasticityPlaneStrain, plasticity.py:430-590): trial stress,
 * sigma_zz = nu (s_xx + s_yy) - E eps_z^p, radial return by the local Newton
 * of plasticity.py:548-560 (tolerance tol, at most max_iter steps), stress,
 * state (q, eps_z^p) and the consistent tangent of plasticity.py:577-588.
 * params [n_elem][4] = (E, nu, sigma_y, H); sigma [nip][n_elem][2][2],
 * state [nip][n_elem][2], tangent [nip][n_elem][16], hgrad = H_inc. */
int fem_plastic_force(const fem_mesh* mesh, const double* params, double tol, int max_iter,
                      const double* v, const uint8_t* con_mask, const double* con_values,
                      int con_mode, const double* sigma_prev, const double* state_prev,
                      const double* de0, double* fe, double* sigma_out, double* state_out,
                      double* tangent, double* hgrad, int32_t* status, void* stream);

/* Vector-Jacobian product of fem_plastic_force at the saved increment inputs
 * (the checkpoint): cotangents of the assembled forces (g), of the stress
 * and state outputs and of hgrad pulled back to sigma_prev, state_prev,
 * thickness and the element field.  Differentiates the return mapping in
 * closed form, which for linear hardening equals differentiating its local
 * Newton iterations. */
int fem_plastic_vjp(const fem_mesh* mesh, const double* params, double tol, int max_iter,
                    const double* v, const uint8_t* con_mask, const double* con_values,
                    int con_mode, const double* sigma_prev, const double* state_prev,
                    const double* de0, const double* g, const double* gsig_out,
                    const double* gstate_out, const double* ghgrad, double* gsig_prev,
                    double* gstate_prev, double* gthick, double* gve, void* stream);

/* ------------------------------------------------------------------------ */
/* Assembly: FEM.assemble_matrix (base.py:398-426).                         */
/* ------------------------------------------------------------------------ */

typedef struct fem_blocks {
  int n_e;                 /* nodes per element */
  int dim;                 /* DOFs per node */
  int64_t n_nod;
  int64_t n_blocks;
  const int64_t* nbr_ptr;  /* [n_nod+1] */
  const int32_t* nbr;      /* [n_blocks] */
  const int64_t* blk_ptr;  /* [n_blocks+1] */
  const int32_t* contrib;  /* [n_elem*n_e*n_e] */
  const int32_t* blk_row;  /* [n_blocks] */
  const int64_t* diag_blk; /* [n_nod] */
  const int64_t* inc_ptr;  /* [n_nod+1] (orphan-node detection) */
} fem_blocks;

/* Scalar CSR values in the reference pattern from Ke (ke_dtype FP64/FP32),
 * summed per slot in ascending element order from +0.0, then constrained
 * rows/columns zeroed and their diagonal set to 1.0 (base.py:410-419). */
int fem_assemble_csr(const fem_blocks* blocks, int ke_dtype, const void* ke,
                     const int64_t* row_ptr, const uint8_t* con_mask, double* val,
                     void* stream);

/* Sliced block layout of the node graph for the FP32 matrix: rows (nodes)
 * in slices of 32, each slice padded to its longest row; block slot k of row
 * a lives at slot sell_base[a/32] + 32 k + a%32 and component c of its
 * dim x dim block at value index sell_base[a/32]*dim^2 + (k dim^2 + c)*32 +
 * a%32.  fem_sell_layout writes sell_base [n_slices+1] and the slot count
 * (*n_slots, host); fem_sell_columns the column of every slot (padding slots
 * point at their own row and hold zeros). */
size_t fem_sell_workspace_bytes(int64_t n_nod);
int fem_sell_layout(const fem_blocks* blocks, int64_t* sell_base, int64_t* n_slots, void* ws,
                    size_t ws_bytes, void* stream);
int fem_sell_columns(const fem_blocks* blocks, const int64_t* sell_base, int32_t* col,
                     void* stream);

/* The same per-slot sums and condensation as fem_assemble_csr, written as
 * FP32 dim x dim blocks into the sliced layout (sval [n_slots * dim^2]). */
int fem_assemble_sell(const fem_blocks* blocks, int ke_dtype, const void* ke,
                      const uint8_t* con_mask, const int64_t* sell_base, int64_t n_slots,
                      float* sval, void* stream);

/* Both copies of the sliced matrix in one pass over FP64 element matrices:
 * sval the FP32 values (each slot's FP64 sum rounded once) and sval64 the
 * FP64 values [n_slots * dim^2] in the same layout.  sval64 serves the
 * mixed solvers' FP64 residual replacements (fem_operator64.sell_val64).
 * No counterpart in the reference, whose solves use one FP64 matrix. */
int fem_assemble_sell_pair(const fem_blocks* blocks, const double* ke, const uint8_t* con_mask,
                           const int64_t* sell_base, int64_t n_slots, float* sval, double* sval64,
                           void* stream);

/* Jacobi: inv_diag[r] = 1 / val[diag_map[r]] (sparse.py:406-407). */
int fem_jacobi(const double* val, const int64_t* diag_map, int64_t n, double* inv_diag,
               int32_t* status, void* stream);

/* Block Jacobi: FP32 inverses [n_nod][dim][dim] of the diagonal blocks of
 * the sliced FP32 matrix. */
int fem_block_jacobi(const fem_blocks* blocks, const float* sval, const int64_t* sell_base,
                     float* inv_blocks, int32_t* status, void* stream);

/* ------------------------------------------------------------------------ */
/* Linear solve: sparse_solve (sparse.py:271-347), Jacobi-CG branch          */
/* (sparse.py:414-421) and the mixed-precision variant.                      */
/* ------------------------------------------------------------------------ */

typedef struct fem_matrix {
  int format;              /* FEM_FMT_CSR_F64 or FEM_FMT_SELL_F32 */
  int block;               /* 1 for CSR, dim for the sliced block layout */
  int64_t n;               /* unknowns */
  int64_t n_rows;          /* scalar rows (CSR) or node rows (sliced) */
  const int64_t* row_ptr;  /* CSR row pointers [n_rows+1] or sell_base [n_slices+1] */
  const int32_t* col;      /* scalar column ids or slot columns */
  const void* val;         /* FP64 [nnz] or FP32 sliced block values */
  const void* precond;     /* FP64 inverse diagonal [n] or FP32 inverse blocks */
} fem_matrix;

typedef struct fem_solve_info {
  int64_t iterations;      /* CG iterations */
  int64_t replacements;    /* FP64 residual replacements (mixed) */
  double rel_residual;     /* ||b - A x|| / ||b|| as tracked by the solver */
  int32_t status;          /* FEM_* */
  double spmv_ms;          /* summed CUDA-event time of the SpMV launches (timing on) */
  int64_t spmv_timed;      /* number of SpMV launches in spmv_ms */
} fem_solve_info;

/* out = a x + b y over nnz stored values of two matrices with one pattern:
 * the Crank-Nicolson system M + dt/2 K of Heat.time_integration
 * (base.py:1519-1521) from the assembled capacity and conductivity values. */
int fem_csr_combine(int64_t nnz, double a, const double* x, double b, const double* y,
                    double* out, void* stream);

/* Crank-Nicolson residual of one time-step Newton iteration
 * (base.py:1486-1495): res = M du + half_dt (f_old + f_int + f_ext), zero
 * where con_mask is set, and sumsq = ||res||^2 (fixed summation order).  M is
 * the assembled FP64 CSR capacity matrix (fem_matrix of format
 * FEM_FMT_CSR_F64); f_old and f_ext are nullable (zero).  ws holds
 * fem_heat_cn_workspace_bytes(M->n) bytes. */
size_t fem_heat_cn_workspace_bytes(int64_t n);
int fem_heat_cn_residual(const fem_matrix* M, const double* du, const double* f_old,
                         const double* f_int, const double* f_ext, double half_dt,
                         const uint8_t* con_mask, double* res, double* sumsq, void* ws,
                         size_t ws_bytes, void* stream);

/* Turns CUDA-event timing of the CG on (1) or off (0).  With the persistent
 * CG (default) spmv_ms covers whole iterations and spmv_timed counts them;
 * with per-iteration kernels it covers the SpMV launches only. */
void fem_set_timing(int enable);

/* CG iteration path: 1 (default) one persistent cooperative kernel per run
 * of iterations, streaming the FP32 3x3 sliced matrix through shared memory
 * with TMA bulk copies; 2 the same kernel with register loads; 0 three
 * kernels per iteration.  Also selectable with the environment variables
 * TORCHFEM_GB300_CG=kernels and TORCHFEM_GB300_TMA=0. */
void fem_set_cg_path(int path);
int fem_get_cg_path(void);

size_t fem_pcg_workspace_bytes(const fem_matrix* A);

/* Preconditioned CG on A x = b from x = 0, stopping at ||r|| <= rtol ||b||
 * (the criterion of cupyx/scipy cg used at sparse.py:417, :508).  FP64 CSR
 * with Jacobi reproduces the reference GPU branch; an FP32 sliced matrix runs
 * the same iteration in single precision. */
int fem_pcg(const fem_matrix* A, const double* b, double* x, double rtol, int64_t max_iter,
            void* ws, size_t ws_bytes, fem_solve_info* info, void* stream);

/* Allocation-free variant of fem_pcg (no counterpart in the reference).
 * For callers that cannot allocate device memory where they solve — a host
 * reaching this library through an FFI with no CUDA allocator binding, or a
 * control loop that cannot accept cudaMalloc's implicit synchronisation or
 * its failure under memory pressure.  Same arguments and results as
 * fem_pcg without (ws, ws_bytes): the scratch is one static 6 MiB device
 * array per GPU, held by every GPU that loads the library until the process
 * exits, so A->n may be at most fem_pcg_static_max_unknowns() (131072);
 * larger systems return FEM_BOUNDS with a message.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and
 * should come before any stream capture on that device; the address is
 * kept for the life of the process, so the entry point must not be used on
 * a device after cudaDeviceReset re-creates its context.  All calls share
 * the array: calls that overlap on the GPU race and must be serialised by
 * the caller.  Nothing from a previous call is reused.  No SpMV event
 * timing (fem_set_timing) is done here, and the timing switch is left as
 * it is. */
int64_t fem_pcg_static_max_unknowns(void);
int fem_pcg_static(const fem_matrix* A, const double* b, double* x, double rtol,
                   int64_t max_iter, fem_solve_info* info, void* stream);

/* FP64 matrix-free operator y = A x of the condensed system: the element
 * kernels apply K to x with constrained entries zeroed, and y = x at
 * constrained DOFs (the matrix assemble_matrix builds, base.py:410-419).
 * sell_val64 (nullable) holds the FP64 values of the same condensed matrix
 * in the sliced layout of the FP32 matrix passed beside the operator
 * (fem_assemble_sell_pair); when set, fem_pcg_mixed and fem_amg_pcg compute
 * their FP64 residuals as one FP64 sliced SpMV over it instead of the
 * element pass.  fem_apply64 always runs the element pass. */
typedef struct fem_operator64 {
  const fem_mesh* mesh;
  const fem_material* mat;
  const uint8_t* con_mask;   /* [n_nod*dim] */
  const double* sell_val64;  /* [n_slots*dim*dim] or NULL */
} fem_operator64;

size_t fem_apply64_workspace_bytes(const fem_operator64* op);
int fem_apply64(const fem_operator64* op, const double* x, double* y, void* ws, size_t ws_bytes,
                void* stream);

/* y = A x in FP64 over the FP64 copy of a sliced matrix
 * (fem_assemble_sell_pair), with the layout of the FP32 sliced
 * matrix A32 (row_ptr = sell_base, col, block): the FP64 residual of the
 * mixed solvers.  Equals fem_apply64 on the same condensed system up to
 * summation order. */
int fem_sell_apply64(const fem_matrix* A32, const double* sval64, const double* x, double* y,
                     void* stream);

size_t fem_pcg_mixed_workspace_bytes(const fem_matrix* A32, const fem_operator64* op);

/* Mixed precision: FP32 sliced-block K and FP32 block-Jacobi CG, with the solution
 * accumulated in FP64 and the recursive residual replaced by the FP64
 * matrix-free residual b - A x whenever it has dropped by `delta` since the
 * last replacement (reliable updates; Sleijpen & van der Vorst 1996).  Stops
 * when the FP64 residual satisfies ||b - A x|| <= rtol ||b||. */
int fem_pcg_mixed(const fem_matrix* A32, const fem_operator64* op, const double* b, double* x,
                  double rtol, double delta, int64_t max_iter, void* ws, size_t ws_bytes,
                  fem_solve_info* info, void* stream);

/* ------------------------------------------------------------------------ */
/* Smoothed-aggregation multigrid (SA-AMG) preconditioner for the FP32       */
/* sliced-block systems: the GPU counterpart of the AMG the reference builds */
/* for its iterative solves, pyamg.smoothed_aggregation_solver(A, B,         */
/* smooth="jacobi") with B = FEM.compute_B() (sparse.py:495-507,             */
/* base.py:316-344), and AmgXSolver on CUDA (amgx.py: create, setup, solve,  */
/* destroy).  Like the AmgX handle, the hierarchy owns its device memory,    */
/* whose size depends on the aggregation: the one exception to the           */
/* no-allocation convention.  fem_amg_destroy frees it.                      */
/* ------------------------------------------------------------------------ */
typedef struct fem_amg fem_amg;

/* Symbolic hierarchy of one mesh and constraint set: aggregation of the
 * node graph (distance-2 independent-set roots), the tentative prolongator
 * from the rigid-body modes of the node coordinates [n_nod][dim] with the
 * constrained components of con_mask [n_nod*dim] (nullable) removed, and
 * the sparsity of every prolongator and coarse operator, down to a coarsest
 * level of at most 96 unknowns.  dim (= blocks->dim) is 2 or 3.  Keeps
 * pointers to blocks->nbr_ptr / nbr, which must outlive the handle. */
int fem_amg_create(const fem_blocks* blocks, const double* coords, const uint8_t* con_mask, fem_amg** out,
                   void* stream);

/* Numeric hierarchy for one FP32 sliced-block matrix of that mesh (A32 with
 * its block-Jacobi inverse in precond, from fem_block_jacobi): spectral
 * estimates of D^-1 A, smoothed prolongators, Galerkin coarse operators,
 * coarse block inverses and the dense coarsest inverse.  A32 must stay
 * unchanged until the next setup. */
int fem_amg_setup(fem_amg* amg, const fem_matrix* A32, void* stream);

/* Keeps the preconditioner of the last fem_amg_setup and makes A32 (a matrix
 * of the same sliced layout, e.g. the next Newton tangent) the operator of
 * the following fem_amg_pcg calls: CG's q = A p and the FP64 refinement use
 * A32, the V-cycle stays the one built for the setup matrix (its FP16
 * smoothing copy, block-Jacobi inverse, Chebyshev bounds and coarse
 * operators), a fixed symmetric positive definite operator, so CG converges
 * to the solution of the new system.  Saves the numeric setup between
 * tangents that change little.  Needs the FP16 smoothing copy
 * (fem_amg_set_half_smoother(1)); FEM_INVALID otherwise.  No counterpart in
 * the reference, which rebuilds its preconditioner per solve. */
int fem_amg_rebind(fem_amg* amg, const fem_matrix* A32);

/* Precision of the level-0 smoothing passes for the setups that follow
 * (process-wide; default 1).  1: the four Chebyshev passes of every V-cycle
 * read an FP16 copy of the level-0 matrix, scaled by a power of two and
 * built by fem_amg_setup (2 bytes per value instead of 4); CG's own product
 * q = A p keeps the FP32 matrix.  The same copy serves pre- and
 * post-smoothing, so the V-cycle stays a fixed symmetric operator.  0: the
 * smoothing passes read the FP32 matrix.  A preconditioner choice with no
 * counterpart in the reference (its AMG runs in FP64). */
void fem_amg_set_half_smoother(int enable);

/* How a V-cycle runs its coarse levels (process-wide; default 1).  1: the
 * restriction from level 0, every coarser level's Chebyshev passes, the
 * coarsest solve and the prolongations back to level 0 run as one
 * cooperative launch whose phases are separated by grid barriers with
 * bounded waits (a wait that runs out ends the solve with FEM_CUDA_ERROR and
 * a "barrier timeout" message).  0, or a device that refuses the
 * cooperative launch: one launch per level operation.  Both keep fixed
 * summation orders, so each is deterministic; they differ only in the order
 * of partial row sums.  No counterpart in the reference. */
void fem_amg_set_fused_cycle(int enable);

/* How the level-0 block SpMVs read the sliced matrix (process-wide; default
 * 1).  1: thread 0 of each slice's CTA streams the slice's slot-rows into a
 * two-stage shared-memory ring with bulk copies (cp.async.bulk completing on
 * mbarriers, waits bounded: a wait that runs out ends the solve with
 * FEM_CUDA_ERROR and a "barrier timeout" message); 0: every thread loads its
 * slot-rows directly.  Same sums in the same order either way.  Scalar rows
 * always use the warp-per-slice kernel.  No counterpart in the reference. */
void fem_amg_set_level0_tma(int enable);

/* Programmatic dependent launch for the CG iteration's chain of kernels
 * (level-0 SpMVs, dot finishers, CG update; process-wide; default 1): each
 * launch may be scheduled while its predecessor drains and waits on the
 * device for the predecessor's completion.  Same work and results.  No
 * counterpart in the reference. */
void fem_amg_set_pdl(int enable);

/* CG preconditioned by one V-cycle (Chebyshev smoothing) on the matrix of
 * the last fem_amg_setup, from x = 0.  With op != NULL: FP64 residual
 * replacement as in fem_pcg_mixed (threshold delta), stopping at
 * ||b - A x|| <= rtol ||b|| in FP64.  With op == NULL: FP32 CG alone,
 * stopping on its recursive residual. */
size_t fem_amg_pcg_workspace_bytes(const fem_amg* amg, const fem_operator64* op);
int fem_amg_pcg(fem_amg* amg, const fem_matrix* A32, const fem_operator64* op, const double* b, double* x,
                double rtol, double delta, int64_t max_iter, void* ws, size_t ws_bytes, fem_solve_info* info,
                void* stream);

void fem_amg_destroy(fem_amg* amg);

/* Read-only view of one level (device pointers owned by the handle). */
typedef struct fem_amg_level {
  int64_t n;                /* block rows */
  int block;                /* block size (dim on level 0, then 6 in 3D / 3 in 2D) */
  int64_t a_nnz;            /* coarse operator blocks (levels >= 1) */
  const int64_t* a_ptr;
  const int32_t* a_col;
  const float* a_val;       /* [a_nnz][block][block] */
  int64_t n_agg;            /* aggregates (0 on the coarsest level) */
  const int32_t* agg;       /* [n] aggregate of each block row, -1 when not aggregated */
  const float* tval;        /* [n][block][K] tentative prolongator rows */
  int64_t p_nnz;
  const int64_t* p_ptr;     /* smoothed prolongator, block CSR [n+1] */
  const int32_t* p_col;
  const float* p_val;       /* [p_nnz][block][K] */
  double rho;               /* spectral estimate of D^-1 A used by the level */
  const float* coarse_inv;  /* coarsest level: dense inverse [n*block]^2 */
  int64_t dropped;          /* near-null modes dropped as dependent (all levels) */
} fem_amg_level;

int fem_amg_levels(const fem_amg* amg);
int fem_amg_level_info(const fem_amg* amg, int level, fem_amg_level* out);

/* Device-to-device copy on the stream (reads handle-owned arrays). */
int fem_copy_device(void* dst, const void* src, size_t bytes, void* stream);

/* Workspace bytes of fem_minres for the FP64 scalar CSR matrix A. */
size_t fem_minres_workspace_bytes(const fem_matrix* A);

/* Jacobi-preconditioned MINRES (Paige-Saunders) from x = 0 on the FP64 CSR
 * matrix (precond = inverse diagonal, fem_jacobi): the reference's GPU
 * method="minres", CuPy's minres with a Jacobi M (sparse.py:405-412).  Stops
 * when the preconditioned residual estimate falls below rtol times its
 * initial value.  Symmetric A (definite or not), positive M. */
int fem_minres(const fem_matrix* A, const double* b, double* x, double rtol, int64_t max_iter, void* ws,
               size_t ws_bytes, fem_solve_info* info, void* stream);

/* Diagnostic of the bounded waits (no counterpart in the reference): one CTA
 * waits at a two-CTA grid barrier that the other CTA never reaches.  The
 * wait gives up after spin_limit clock cycles and the call returns
 * FEM_CUDA_ERROR with the barrier-timeout message; the context stays usable.
 * ws: fem_diag_workspace_bytes() bytes of device memory. */
size_t fem_diag_workspace_bytes(void);
int fem_diag_barrier_timeout(void* ws, size_t ws_bytes, long long spin_limit, void* stream);

/* ------------------------------------------------------------------------ */
/* Modal analysis (FEM.solve_modes, base.py:1097-1129; eigen-solve          */
/* sparse.py:798-1011).                                                      */
/* ------------------------------------------------------------------------ */

/* Element mass matrices me [n_elem][n_e d][n_e d] of a mechanics model:
 * sum_ip w detJ rho t N N^T expanded to the d DOFs of each node (Kronecker
 * product with I_d), rho [n_elem], t the mesh thickness (1 when NULL), nval
 * [nip][n_e] the shape-function values at the integration points.  Replaces
 * FEM.integrate_mass (base.py:376-396) with compute_m (solid.py:60-62,
 * planar.py:94-96). */
int fem_mass_matrices(const fem_mesh* mesh, const double* rho, const double* nval, int d, double* me,
                      void* stream);

/* Y = A X for a scalar FP64 CSR matrix and row-major blocks X, Y
 * [n][nvec] of device memory: the operator applications of the block
 * eigensolver that replaces the reference's shift-invert eigsh on the free
 * DOFs (sparse.py:798-827). */
int fem_csr_spmm(const fem_matrix* A, int nvec, const double* X, double* Y, void* stream);

/* ------------------------------------------------------------- assembly --
 * Parts coupled by kinematic constraints (Assembly.solve,
 * assembly.py:378-650): the coupling map T [n_dofs x n_retained] eliminates
 * the secondary DOFs, u = T q, and the solved system is
 * K_r = T^T blockdiag(K_parts) T with the Dirichlet condensation of
 * Assembly._stiffness (assembly.py:295-334).  The host builds the pattern of
 * K_r and, per entry, the contributing part-matrix entries once per solve.
 *
 * Values of K_r: out[e] = sum_{c in [ptr[e], ptr[e+1])} coef[c] * kval[src[c]]
 * (kval: the parts' FP64 CSR values, concatenated; coef: the product of the
 * two T coefficients), summed in list order; then fix[e] = 1 zeroes the entry
 * (a constrained row or column) and fix[e] = 2 sets it to 1 (a constrained
 * diagonal).  fix may be NULL.  Replaces torch.sparse.mm(T^T, K T) and the
 * condensation of Assembly._stiffness. */
int fem_coupled_values(int64_t n_out, const int64_t* ptr, const int64_t* src, const double* coef,
                       const double* kval, const uint8_t* fix, double* out, void* stream);

/* y = A x for a rectangular FP64 CSR matrix [n_rows x any] with int64 row
 * pointers and int32 columns: u = T q and T^T (F_int - F_ext) of an assembly
 * (the _mv products of assembly.py:23-25). */
int fem_csr_apply(int64_t n_rows, const int64_t* row_ptr, const int32_t* col, const double* val,
                  const double* x, double* y, void* stream);

/* ---------------------------------------------------------------- shell --
 * Tria1 flat-facet shell, homogeneous linear-elastic section (the reference's
 * Shell with a plane-stress material, src/torchfem/shell.py:48-603).  Nodes
 * carry (u, v, w, rx, ry, rz); element DOFs are node-major, 18 per element. */
typedef struct fem_shell {
  int64_t n_nod;
  int64_t n_elem;
  const double* nodes;        /* [n_nod][3] */
  const int32_t* elements;    /* [n_elem][3] */
  const double* orientation;  /* [n_elem][3] material reference direction, NULL = global x */
  const double* thickness;    /* [n_elem] */
  int n_z;                    /* through-thickness stations (odd, Simpson) */
  const double* z;            /* [n_z] station positions / thickness, in [-1/2, 1/2] */
  const double* w;            /* [n_z] station weights / thickness, summing to one */
  double kappa;               /* transverse shear correction factor */
  double nu_t;                /* Poisson's ratio of the transverse shear scaling */
  double drill;               /* drilling-rotation penalty */
} fem_shell;

/* Element matrices ke [n_elem][18][18] (global axes) of the shell with per-
 * element material data mat [n_elem][11] = (plane-stress tangent in Voigt
 * form, row-major 3x3; transverse shear moduli G_xz, G_yz).
 * Replaces Shell.integrate_material's stiffness (shell.py:456-586) with the
 * frames of Shell.eval_shape_functions (shell.py:358-387) and the strain
 * operators _Dm/_Db/_Ds (shell.py:263-356). */
int fem_shell_stiffness(const fem_shell* shell, const double* mat, double* ke, int32_t* status, void* stream);

/* Element forces fe [n_elem][18] = ke u_e of the total nodal DOFs u
 * [n_nod][6], and optionally the station stresses [n_z][n_elem][2][2]
 * (local axes) of u from zero prestress (shell.py:474-504, 588-603). */
int fem_shell_force(const fem_shell* shell, const double* mat, const double* ke, const double* u, double* fe,
                    double* stress, void* stream);

/* Vector-Jacobian product of (assembled forces, station stresses) with the
 * nodal force cotangent a [n_nod][6] (may be NULL) and the stress cotangent
 * gstress [n_z][n_elem][2][2] (may be NULL): gradients for mat
 * [n_elem][11], thickness [n_elem] and the stress part of the element-DOF
 * gradient gue [n_elem][18] (each output may be NULL).  Replaces the autograd
 * replay of Shell.integrate_material inside NewtonRaphsonAdjoint
 * (sparse.py:690-705). */
int fem_shell_vjp(const fem_shell* shell, const double* mat, const double* u, const double* a,
                  const double* gstress, double* gmat, double* gthick, double* gue, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TORCHFEM_GB300_H */
