/*
 * gales_asm.h — C ABI of the GB300 assembly library for the compressible
 * multicomponent fluid_mc equations of GALES-multi-fluid.
 *
 * One call fills the global CSR tangent matrix A and the right-hand side b of
 * one Newton iteration, exactly what the reference's
 *   fluid_assembly<fluid<ic_bc,dim>, scatter<dofs_ic_bc>, dim>::execute()
 * (sim/fluid_mc/P0/fluid_assembly.hpp:39-68) fills into its Epetra
 * linear_system (src/fem/ls/linear_system.hpp:35-105).  The element-level
 * plugin points of the reference (fluid::execute_i / execute_b,
 * sim/fluid_mc/P0/fluid_2d.hpp:171,209, and scatter::execute,
 * src/fem/ls/scatter.hpp:37) are too fine-grained for a GPU, so the whole
 * assembly driver is the replaced unit.
 *
 * Conventions (all taken from the reference):
 *   - dofs per node nd = 2 + dim + nb_comp - 1, ordered
 *     (p, v_1..v_dim, T, Y_1..Y_{nb_comp-1})        (main.cpp:82, fluid_2d.hpp:86-92)
 *   - nodal state is AoS FP64, index node*nd + k; slot I = current iterate,
 *     slot P = previous time level                 (dof_state.hpp:43-49)
 *   - global dof id = node*nd + k                   (node.hpp:73)
 *   - the matrix is scalar CSR with sorted global column ids per row; every
 *     element contributes a dense (nen*nd)^2 block (linear_system.hpp:46-63)
 *   - b = -R (the element returns r = -r_, fluid_2d.hpp:200-201) and
 *     Dirichlet rows are replaced as in scatter.hpp:62-78.
 *
 * Errors: every entry point returns an int status (0 = OK, otherwise an OR of
 * GALES_ERR_* bits).  Kernels never trap; a device status word records the
 * first offending element.  The reference aborts through MPI_Abort instead
 * (src/fem/base/algorithm.hpp:37-44).
 *
 * Pointers passed to assemble/residual/vjp may be host or device memory; the
 * library detects which with cudaPointerGetAttributes.  A handle is
 * single-threaded and stream-ordered; distinct handles are independent.
 */
#ifndef GALES_ASM_H_
#define GALES_ASM_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GALES_MAX_DIM 3
#define GALES_MAX_COMP 8
#define GALES_MAX_ND (2 + GALES_MAX_DIM + GALES_MAX_COMP - 1)
#define GALES_MAX_FLAGS 32

/* status bits */
#define GALES_OK 0
#define GALES_ERR_BAD_INPUT 1
#define GALES_ERR_NEG_JACOBIAN 2   /* quad.hpp:215-218, 549-552 */
#define GALES_ERR_SINGULAR 4       /* algorithm.hpp:406-410 (LU of DUDY) */
#define GALES_ERR_NONFINITE 8
#define GALES_ERR_CUDA 16
#define GALES_ERR_UNSUPPORTED 32
#define GALES_ERR_NO_MEMORY 64
#define GALES_ERR_MAGMA 128        /* a magma property outside its lookup tables or a zero
                                      viscosity denominator (mixtures.hpp:342-412,
                                      GiordanoEtAlViscosityModel.hpp; the reference stops) */
#define GALES_ERR_TIMEOUT 256      /* a bounded device wait (a bulk copy of point records) ran
                                      out; not expected on a working device */

/* numerical forms */
#define GALES_FORM_FP64 0    /* every operation in FP64 (the reference's arithmetic) */
#define GALES_FORM_MIXED 1   /* FP32 element integrals; FP64 EOS, tau, accumulation */

/* chemical kinds (src/fem/physical_props/fluid/chemicals.hpp) */
#define GALES_CH_CUSTOM 0     /* custom_chemical, chemicals.hpp:19-49 */
#define GALES_CH_IDEAL_GAS 1  /* ideal_gas, chemicals.hpp:198-271 */

/* stabilisation parameter variants (fluid_2d.hpp:877-1022) */
#define GALES_TAU_NONE 0
#define GALES_TAU_NON_DIAG_COMP_2001 2001
#define GALES_TAU_NON_DIAG_COMP_2019 2019
#define GALES_TAU_DIAG_INCOMP_2007 2007
#define GALES_TAU_DIAG_2014 2014

/* VJP modes */
#define GALES_VJP_EXACT 0    /* lambda^T dB/dI of the assembled rhs, all coefficients differentiated */
#define GALES_VJP_FROZEN 1   /* A^T lambda with the frozen-coefficient tangent A */

/* scatter strategies */
#define GALES_SCATTER_ATOMIC 0
#define GALES_SCATTER_COLOURED 1

/* Mesh on one rank.  Node ids are 0..n_nodes-1 and equal the node gid.
 * Element node order and side numbering follow element.hpp:63-176 (2D) and
 * element.hpp:360-477 (3D).  Supported (dim, nen): (2,3) tri, (2,4) quad,
 * (3,4) tet, (3,8) hex. */
typedef struct gales_mesh_desc {
  int32_t dim;
  int32_t nen;
  int64_t n_nodes;
  int64_t n_elements;
  const double* coords;          /* [n_nodes][dim] */
  const int32_t* conn;           /* [n_elements][nen] */
  const int32_t* node_flag;      /* [n_nodes], node.hpp flag (0 interior) */
  const uint8_t* el_on_boundary; /* [n_elements], element flag > 0 (mesh.hpp:224-225); NULL = none */
  int64_t n_bd_sides;            /* sides with side flag > 0 (mesh.hpp:409-446) */
  const int32_t* bd_side_el;     /* [n_bd_sides] element index */
  const int32_t* bd_side_local;  /* [n_bd_sides] local side index of that element */
  const int32_t* bd_side_flag;   /* [n_bd_sides] side flag (1..GALES_MAX_FLAGS-1) */
} gales_mesh_desc;

/* Stored constants of one chemical after construction (base_chemical.hpp:80-90).
 * custom: rho, mu, cp, kappa, alpha, beta are constants; cv is derived per call
 *         as cp - T*alpha^2/(rho*beta) (cp if beta == 0), c = 1/sqrt(rho*beta).
 * ideal gas: R (specific gas constant), gamma, cv, cp, mu, kappa are constants;
 *         rho = p/(R T), beta = 1/p, alpha = 1/T, c = sqrt(gamma R T). */
typedef struct gales_chemical_desc {
  int32_t kind;
  int32_t reserved;
  double rho, mu, cp, cv, kappa, alpha, beta;
  double R, gamma;
  double chemical_diffusivity; /* base_chemical.hpp:86 default 1e-10 */
} gales_chemical_desc;

/* mix_of_ch mixture (fluid_properties.hpp:199-227) */
typedef struct gales_material_desc {
  int32_t nb_comp;
  int32_t reserved;
  gales_chemical_desc comp[GALES_MAX_COMP];
} gales_material_desc;

/* Neumann / prescribed mass flux data of one side flag, the data form of the
 * policy calls fluid_ic_bc::neumann_* and mass_flux* (fluid_ic_bc.hpp:133-211)
 * consumed by fluid_2d.hpp:610-868.  Stress override tau_kj (k <= j) is bit
 * k*3+j of tau_mask with value tau[k*3+j]; heat flux q_k is bit k; species
 * flux J_k of component i is bit k*8+i; mass flux rho*v_k is bit k. */
typedef struct gales_side_bc {
  uint32_t tau_mask;
  uint32_t q_mask;
  uint32_t J_mask;
  uint32_t mass_flux_mask;
  double tau[9];
  double q[3];
  double J[3][8];
  double mass_flux[3];
} gales_side_bc;

/* Run-time flags (read_setup.hpp; sim/fluid_mc/P0/setup.txt:24-31) plus the
 * ic_bc policy as data. */
typedef struct gales_setup_desc {
  int32_t tau;            /* GALES_TAU_* */
  int32_t dc_2006;        /* discontinuity capturing on/off */
  int32_t steady_state;
  int32_t reserved;
  double dc_sharp;        /* 1, 1.5 or 2 (fluid_2d.hpp:1055-1057) */
  double dc_scale_fact;
  double gravity[3];      /* fluid_ic_bc::body_force, fluid_ic_bc.hpp:44-56 */
  double p_ref, T_ref;    /* dc_2006 reference state, fluid_ic_bc.hpp:33 */
  double v_ref[3];
  /* per node flag: bit k set = dof k Dirichlet-constrained
   * (fluid_dofs_ic_bc::dof_constraint, fluid_dofs_ic_bc.hpp:86-117) */
  uint32_t dirichlet_mask[GALES_MAX_FLAGS];
  gales_side_bc side_bc[GALES_MAX_FLAGS];
} gales_setup_desc;

typedef struct gales_asm gales_asm;

/* Fill a chemical descriptor the way the reference constructors do. */
void gales_chemical_custom(gales_chemical_desc* c, double rho, double mu, double cp, double kappa,
                           double alpha, double beta);               /* chemicals.hpp:23-33 */
void gales_chemical_ideal_gas(gales_chemical_desc* c, double molar_mass, double gamma); /* chemicals.hpp:237-246 */
/* Defaults of the shipped case: tau 2019, dc_2006 on, dc_sharp 2, scale 1,
 * unsteady, gravity (0,-9.81) in 2D and 0 in 3D, p_ref 70e6, T_ref 1300,
 * v_ref 0, no Dirichlet, no Neumann overrides. */
void gales_setup_default(gales_setup_desc* s, int32_t dim);

/* Create a handle: uploads the mesh, builds the CSR graph (linear_system.hpp:40-66),
 * the element colouring and the per-element CSR slot table.  Replaces
 * linear_system's constructor and fluid's constructor (u_ref_inv, fluid_2d.hpp:123-135). */
int gales_asm_create(const gales_mesh_desc* mesh, const gales_material_desc* mat,
                     const gales_setup_desc* setup, int device, gales_asm** out);
void gales_asm_destroy(gales_asm* h);

/* CSR pattern on the host (owned by the handle): n_rows = n_nodes*nd,
 * row_ptr[n_rows+1] (int64), col[nnz] (int32, sorted per row). */
int gales_asm_pattern(gales_asm* h, int64_t* n_rows, int64_t* nnz, const int64_t** row_ptr,
                      const int32_t** col);
/* Node-level graph (the CSR is this graph with every entry expanded to an nd x nd block). */
int gales_asm_node_graph(gales_asm* h, int64_t* n_nodes, int64_t* nnz_nodes,
                         const int64_t** node_row_ptr, const int32_t** node_col);
/* Greedy element colouring: no two elements of one colour share a node. */
int gales_asm_colouring(gales_asm* h, int32_t* n_colours, const int32_t** colour);
int gales_asm_set_scatter(gales_asm* h, int32_t mode); /* GALES_SCATTER_* */
/* Elements per chunk of the interior pass (rounded down to a multiple of 4, at least 4,
 * at most the chunk the handle's record buffer was sized for: as many elements as 3 GiB
 * of point records hold); 0 restores that default.  Each chunk runs the point kernel,
 * then the matrix kernel.  No counterpart in the reference (its assembly has no
 * chunks); smaller chunks cost launch tails, the results are the same. */
int gales_asm_set_chunk(gales_asm* h, int64_t elements);

/* One assembly: vals[nnz] and rhs[n_rows] are overwritten (linear_system::clear
 * is part of the call, linear_system.hpp:90-94).  stream: cudaStream_t or NULL. */
int gales_asm_assemble(gales_asm* h, const double* I, const double* P, double dt, int32_t form,
                       double* vals, double* rhs, void* stream);
/* Assembly that allocates nothing (no counterpart in the reference).  For callers
 * that must not allocate device memory during the call: programs whose device
 * memory belongs to another allocator or to a fixed quota, and loops that keep a
 * fixed memory footprint after set-up.  Same result as gales_asm_assemble, but
 * I, P, vals and rhs must be device pointers (host buffers are rejected with
 * GALES_ERR_BAD_INPUT since staging them would allocate), the work runs on the
 * caller's stream only, and the per-point records live in one library-wide
 * device array of GALES_NOALLOC_SCRATCH_BYTES, which every GPU that loads the
 * library keeps until exit.  Point records are laid out in blocks of up to four
 * elements: when four elements' records exceed that size the call is rejected with
 * GALES_ERR_UNSUPPORTED; larger meshes are processed in chunks of a multiple of four
 * elements.
 * The first call on a device looks up the array's device address (once per
 * device) and keeps it for the life of the process; make that first call before any
 * stream capture.  A reset of the device (cudaDeviceReset, or any reset of its
 * primary context) frees every handle's device memory and leaves that address
 * stale: do not use the library on a device after resetting it.  All calls, from every
 * handle, share the one array and it keeps the last call's contents: calls that
 * overlap on the GPU (concurrent streams or threads) race on it, so order them. */
#define GALES_NOALLOC_SCRATCH_BYTES (8u << 20)
int gales_asm_assemble_noalloc(gales_asm* h, const double* I, const double* P, double dt, int32_t form,
                               double* vals, double* rhs, void* stream);
/* Enqueue one assembly on `stream` and return: device pointers only, no host
 * synchronisation, no timing events and no allocation, so a sequence of calls can be
 * captured into a CUDA graph and replayed (e.g. the Newton iterations of one time
 * step).  vals may be NULL (residual only).  Errors found by the kernels accumulate
 * in the status word until gales_asm_sync.  No reference counterpart: the reference
 * assembles synchronously (fluid_assembly.hpp:39-68). */
int gales_asm_enqueue(gales_asm* h, const double* I, const double* P, double dt, int32_t form, double* vals,
                      double* rhs, void* stream);
/* Wait for `stream`, return the status of the work enqueued since the last sync
 * (0 or error bits, first offending element via gales_asm_status) and clear it. */
int gales_asm_sync(gales_asm* h, void* stream);
/* Residual only (rhs), no matrix. */
int gales_asm_residual(gales_asm* h, const double* I, const double* P, double dt, int32_t form,
                       double* rhs, void* stream);
/* Vector-Jacobian product of the assembled rhs b(I; theta):
 *   g_state[n_rows]  = (db/dI)^T lambda           (mode EXACT)
 *                    = A^T lambda                  (mode FROZEN, A the assembled tangent)
 *   g_params[3*nb_comp] = (db/dtheta)^T lambda, theta_c = (density parameter, mu, cp) of
 *                    component c (density parameter = rho for custom chemicals, molar mass
 *                    for ideal gases).  Only in mode EXACT; may be NULL. */
int gales_asm_vjp(gales_asm* h, const double* I, const double* P, double dt, const double* lambda,
                  int32_t mode, double* g_state, double* g_params, void* stream);
/* Element-level blocks, the batched form of the reference's integral plugin call
 *   fluid::execute_i(el, dofs, m, r)   (which = 0, fluid_2d.hpp:171-202)
 *   fluid::execute_b(el, dofs, m, r)   (which = 1, fluid_2d.hpp:209-245)
 * for the n listed elements: m_out[n][(nen*nd)^2] (row-major, row nd*b+jb) and
 * r_out[n][nen*nd] with r = -r_, before Dirichlet rows and scatter.  m_out may be
 * NULL (residual only).  elements is a host array. */
int gales_asm_element_blocks(gales_asm* h, const double* I, const double* P, double dt, int32_t form,
                             int32_t which, const int32_t* elements, int64_t n, double* m_out,
                             double* r_out, void* stream);
/* ||b||_2 of a rhs vector (residual_check.hpp:48-51). */
int gales_asm_norm2(gales_asm* h, const double* rhs, double* out, void* stream);

/* Adaptive time step of the multicomponent solver (adaptive_time_criteria::f_mc,
 * adaptive_time_step.hpp:183-260, called from main.cpp:258-261 after a time step): for
 * every element the smallest over its Gauss points of CFL/use, with
 * use = 2 max(2 mu/rho, kappa/(rho cv))/h^2 + v_tau/h from the state I (FP64, the
 * reference's operations), or 1.2 dt where |v| < DBL_EPSILON.  dt_el (n_elements,
 * host or device, may be NULL) receives those values; *dt_new the next step by
 * set_dt (380-393; gales_dt_update).  The call synchronises its stream. */
int gales_asm_adaptive_dt(gales_asm* h, const double* I, double dt, double cfl, double dt_min, double dt_max,
                          double* dt_el, double* dt_new, void* stream);
/* set_dt (adaptive_time_step.hpp:380-393) on the smallest element value: at most
 * 1.01 dt, then clamped to [dt_min, dt_max].  Host arithmetic only. */
double gales_dt_update(double dt_elem_min, double dt, double dt_min, double dt_max);

/* Secondary variables at the nodes (secondary_dofs::execute, secondary_dofs.hpp:56-101,
 * the mixture of every node's state at shear rate 0): out[f * n_nodes + node] for
 * f = 0..7 = rho, mu, cp, cv, alpha, beta, kappa, sound speed (host or device, 8 n_nodes
 * doubles).  The magma volume and mass fractions of the same routine (pp_vf_g) come
 * from gales_asm_magma_fractions.  The call synchronises its stream. */
int gales_asm_secondary_dofs(gales_asm* h, const double* I, double* out, void* stream);

/* Hydrostatic pressure column of the multicomponent solver (pressure_profile_mc,
 * pressure_profile.hpp:326-516, Runge_Kutta 480-496), host arithmetic: from p_out[0] = p0
 * at the top, p_out[i+1] = p_out[i] + h/6 (m1 + 2 (m2 + m3) + m4) with m = 9.81 rho(p, T,
 * Y) at the start (T[i], Y[i]), twice at the midpoint (T1[i], Y1[i]) and at the end
 * (T[i+1], Y[i+1]).  T and Y sample the case's initial_T / initial_Y at the column points
 * y_i = max - h i, T1 and Y1 at y_i - h/2 (n_steps + 1 entries each; Y holds the nc - 1
 * independent fractions per point, the last is 1 - their sum as the reference forms it).
 * p_out has n_steps + 1 entries. */
int gales_pressure_profile(const gales_material_desc* mat, double p0, double h, int32_t n_steps, const double* T,
                           const double* T1, const double* Y, const double* Y1, double* p_out);
/* p_interpolation (pressure_profile.hpp:26-41): linear interpolation of the column
 * (y_col, p_col) at the heights y[0..n); GALES_ERR_BAD_INPUT when a height falls
 * outside the column (where the reference stops with an error). */
int gales_pressure_interpolate(const double* y_col, const double* p_col, int32_t n_col, const double* y, int64_t n,
                               double* p_out);

/* Linear solve of the assembled system on the GPU, replacing belos_linear_solver
 * (src/fem/ls/belos_linear_solver_factory.hpp:69-274) as main.cpp:216-245 drives it:
 * flexible GMRES with a right ILU(fill) preconditioner (Belos "Flexible GMRES", Ifpack
 * "ILU", setup.txt ls_* keys), x0 = 0, converged when ||b - A x|| <= rel_res_tol ||b||.
 * The factor is the scalar ILU(fill) of the assembled CSR matrix, stored as node blocks
 * (the pattern's dense nd x nd blocks make the two identical).  One solver per assembly
 * handle; it reads the handle's node graph at creation. */
#define GALES_PRECOND_NONE 0
#define GALES_PRECOND_ILU 1       /* FP64 factor: the scalar ILU(fill) bit for bit */
#define GALES_PRECOND_ILU_FP32 2  /* the same factorisation and substitutions in FP32 (the
                                     Krylov vectors, products and residuals stay FP64) */

typedef struct gales_solver_params {
  double rel_res_tol;    /* ls_rel_res_tol (belos_linear_solver_factory.hpp:77) */
  int32_t maxsubspace;   /* ls_maxsubspace: Krylov vectors per cycle ("Num Blocks") */
  int32_t maxrestarts;   /* ls_maxrestarts */
  int64_t maxiters;      /* ls_maxiters; -1: rows - 1 (belos_linear_solver_factory.hpp:128) */
  int32_t fill;          /* ls_fill: ILU level of fill */
  int32_t precond;       /* GALES_PRECOND_ILU (ls_precond ILU), _ILU_FP32 or _NONE */
} gales_solver_params;

typedef struct gales_solver_result {
  int64_t iterations;    /* num_it(): Arnoldi steps over all cycles */
  double abs_res;        /* ARE(): ||b - A x|| */
  double rel_res;        /* RRE(): ||b - A x|| / ||b|| */
  double seconds;        /* wall time of the call (execute()'s return value) */
  int32_t converged;
  int32_t cycles;        /* GMRES cycles (1 + restarts) */
} gales_solver_result;

typedef struct gales_solver gales_solver;

/* The shipped settings (sim/fluid_mc/P0/setup.txt:10-16): 1e-9, 200, 5, -1, fill 1, ILU. */
void gales_solver_default(gales_solver_params* p);
/* Symbolic factorisation and level sets on the device's current context; p may be NULL
 * (defaults).  Allocates the factor and (maxsubspace + 1) + maxsubspace Krylov vectors. */
int gales_solver_create(gales_asm* h, const gales_solver_params* p, gales_solver** out);
/* execute(): factorises vals (the handle's CSR values), then solves A x = rhs.  vals,
 * rhs and x are host or device arrays; the call synchronises its stream.  res may be
 * NULL.  GALES_ERR_SINGULAR for a zero pivot in the factorisation. */
int gales_solver_solve(gales_solver* s, const double* vals, const double* rhs, double* x, gales_solver_result* res,
                       void* stream);
/* The factorisation alone (synchronises), and z = M^-1 v with the current factor
 * (device arrays, enqueued on the stream). */
int gales_solver_factorize(gales_solver* s, const double* vals, void* stream);
int gales_solver_apply(gales_solver* s, const double* v, double* z, void* stream);
/* The factor as node blocks: the block pattern (host arrays owned by the solver) and,
 * when vals is not NULL, nnz_blocks * nd * nd values (block-major, row-major blocks;
 * unit L strictly below the diagonal, U on and above it).  Synchronises the device. */
int gales_solver_factor(gales_solver* s, int64_t* n_block_rows, int64_t* nnz_blocks, const int64_t** row_ptr,
                        const int32_t** col, double* vals);
/* Number of levels of the forward and backward substitutions (launches per sweep). */
int gales_solver_levels(gales_solver* s, int32_t* n_levels_fwd, int32_t* n_levels_bwd);
/* fluid_updater::corrector and model::dof_trimmer (fluid_updater.hpp:23-26,
 * model.hpp:176-184): I += dx on the device, then every node's dofs with index in
 * [trim_first, trim_last) clamped to max(lo, min(v, hi)) (main.cpp:235 trims dof 4 to
 * [0, 1]).  Device arrays, enqueued on the stream. */
int gales_solver_correct(gales_solver* s, double* I, const double* dx, int32_t trim_first, int32_t trim_last,
                         double lo, double hi, void* stream);
int64_t gales_solver_launches(gales_solver* s);
const char* gales_solver_last_error(gales_solver* s);
void gales_solver_destroy(gales_solver* s);
/* Host-only: the node-level ILU(fill) pattern (sorted columns, diagonal included) of a
 * graph with sorted columns, and each row's forward / backward substitution level.
 * With f_row_ptr NULL only *nnz is set.  n_levels (may be NULL) receives the two level
 * counts.  No GPU use. */
int gales_iluk_pattern(int64_t n, const int64_t* row_ptr, const int32_t* col, int32_t fill, int64_t* nnz,
                       int64_t* f_row_ptr, int32_t* f_col, int32_t* level_fwd, int32_t* level_bwd,
                       int32_t* n_levels);

/* Magma mixtures (src/fem/physical_props/fluid/mixtures.hpp:114-511): melt, H2O(l),
 * CO2(l), H2O(g), CO2(g) with the liquid-phase volatile fractions from solubility lookup
 * tables, Giordano et al. (2008) viscosity (GiordanoEtAlViscosityModel.hpp) and the gas
 * and crystal corrections of mixtures.hpp:250-341; several magmas form a mixture of
 * sub-mixtures (fluid_properties.hpp:171-200, props.txt "mix_of_mix" of "magma_mix"). */
#define GALES_GAS_MU_NONE 0
#define GALES_GAS_MU_ISHII_ZUBER 1        /* mixtures.hpp:296-299 */
#define GALES_GAS_MU_PAL_2003 2           /* mixtures.hpp:260-291 (Newton loop bounded to 200 steps) */
#define GALES_CRYSTAL_MU_NONE 0
#define GALES_CRYSTAL_MU_EINSTEIN_ROSCOE 1  /* mixtures.hpp:305-308 */
#define GALES_CRYSTAL_MU_CARICCHI 2         /* mixtures.hpp:314-330 */
/* sub-mixture kinds of a mix_of_mix (fluid_properties_reader.hpp:17, 127-141) */
#define GALES_SUBMIX_MAGMA 0      /* magma_mix (mixtures.hpp:114-511) */
#define GALES_SUBMIX_CUSTOM 1     /* custom_mix: constant properties (mixtures.hpp:69-101) */
#define GALES_SUBMIX_CHEMICAL 2   /* ch_as_mix: one chemical as a sub-mixture (mixtures.hpp:25-53) */
/* magma status bits (gales_magma_status) */
#define GALES_MAGMA_LOOKUP_RANGE 1   /* a pressure or temperature outside the table (the reference stops) */
#define GALES_MAGMA_VISCOSITY 2      /* a zero denominator of the viscosity model (the reference stops) */
#define GALES_MAGMA_PAL_ITER 4       /* Pal 2003's iteration did not stop within 200 steps */

/* One magma_mix block of props.txt (fluid_properties_reader.hpp:293-420; defaults there:
 * melt_kappa 1.5, h2o_l/co2_l cp 2278, kappa 0.64).  The solubility tables are the files
 * of input/lookuptable: pressures (equispaced, n_p), optional temperatures (n_T > 0:
 * bilinear in (T, p), tables [n_T][n_p]; n_T = 0: linear in p, tables [n_p]), and the
 * weight fractions of H2O and CO2 dissolved in the liquid.  Host arrays, copied at
 * creation. */
typedef struct gales_magma_desc {
  double oxide_wf[10];   /* SiO2 TiO2 Al2O3 Fe2O3 FeO MnO MgO CaO Na2O K2O (normalised) */
  double melt_kappa;
  double h2o_wf, h2o_l_cp, h2o_l_kappa;
  double co2_wf, co2_l_cp, co2_l_kappa;
  double crystal_fraction, crystal_rho;
  int32_t gas_on_mu;      /* GALES_GAS_MU_* */
  int32_t crystal_on_mu;  /* GALES_CRYSTAL_MU_* */
  int32_t n_p, n_T;
  const double* p_table;
  const double* T_table;
  const double* wf_l_h2o;
  const double* wf_l_co2;
  /* The kind of this sub-mixture (GALES_SUBMIX_*; 0 = magma_mix, which reads the fields
   * above).  custom_mix reads rho, mu, cp, kappa, alpha and beta of `chemical`
   * (kind GALES_CH_CUSTOM); ch_as_mix reads `chemical` (a custom chemical or an ideal
   * gas).  Neither copies the chemical's diffusivity: theirs stays base_chemical's
   * 1e-10 (base_chemical.hpp:86), and their gas fractions (pp_vf_g) are 0. */
  int32_t kind;
  int32_t reserved;
  gales_chemical_desc chemical;
} gales_magma_desc;

typedef struct gales_magma gales_magma;

/* Upload nb_comp sub-mixtures (1..GALES_MAX_COMP; magma_mix, custom_mix or ch_as_mix)
 * to the current device. */
int gales_magma_create(const gales_magma_desc* comps, int32_t nb_comp, gales_magma** out);
/* Mixture-of-magmas properties at n points (p[i], T[i], all nb_comp mass fractions
 * Y[i * nb_comp + c], shear rate shear[i] or NULL = 0), one GPU thread per point:
 * out[f * n + i] for f = rho, mu, cp, cv, kappa, sound speed, alpha, beta; comp (may be
 * NULL) [(c * 4 + k) * n + i] for k = rho_c, e_c = cv_c T, chemical diffusivity, gas
 * volume fraction of magma c.  Host or device arrays; synchronises the stream.  Returns
 * 0, or GALES_ERR_BAD_INPUT with the GALES_MAGMA_* bits in gales_magma_status. */
int gales_magma_properties(gales_magma* m, const double* p, const double* T, const double* Y, const double* shear,
                           int64_t n, double* out, double* comp, void* stream);
int gales_magma_status(gales_magma* m);
const char* gales_magma_last_error(gales_magma* m);
void gales_magma_destroy(gales_magma* m);
/* Attach magma mixtures as the assembly's material (m == NULL detaches them): from then
 * on the handle's assembly, residual, frozen VJP, element blocks, adaptive time step and
 * secondary variables evaluate every point's properties with fluid_properties'
 * mix_of_mix of magma_mix (fluid_properties.hpp:171-200), at P with shear rate 0 and at
 * I and the boundary points with the point's shear rate (fluid_2d.hpp:186, 193-194,
 * 234-235; compute_shear_rate, non_newtonian.hpp:23-39), instead of the chemicals given
 * at creation; u_ref_inv is recomputed from the magmas (fluid_2d.hpp:123-135).  The
 * reference selects this with props.txt's "mix_of_mix" (fluid_properties_reader.hpp).
 * m must have the handle's number of components, live on its device and outlive the
 * attachment.  A point outside a magma's lookup tables sets GALES_ERR_MAGMA (the
 * reference stops).  The exact VJP returns GALES_ERR_UNSUPPORTED while magmas are
 * attached.  Call outside any stream capture. */
int gales_asm_set_magma(gales_asm* h, gales_magma* m);
/* The gas fractions of secondary_dofs::execute with pp_vf_g (secondary_dofs.hpp:56-131)
 * at every node's state I (shear rate 0), with magmas attached: out[f * n_nodes + node]
 * for f = vf_g_comp_c, vf_comp_c (c = 0..nb_comp-1, interleaved), then vf_g_on_total,
 * vf_h2o_g_on_total, vf_co2_g_on_total, wf_g_on_total, wf_h2o_g_on_total,
 * wf_co2_g_on_total: 2 nb_comp + 6 fields.  Host or device buffers. */
int gales_asm_magma_fractions(gales_asm* h, const double* I, double* out, void* stream);

/* Status of the last call: error bits and the first offending element (-1 if none). */
int gales_asm_status(gales_asm* h, int64_t* first_bad_element);
const char* gales_asm_last_error(gales_asm* h);
/* Device time in ms of the last assemble/residual/vjp call (CUDA events on its stream). */
double gales_asm_last_ms(gales_asm* h);
/* Device time in ms of one phase of the last assemble/residual call, CUDA events on
 * its stream: 0 = clearing A and b, 1 = interior element kernel(s), 2 = boundary pass,
 * 3 / 4 = the point / matrix stage of the interior pass's first chunk (the whole pass
 * when it has one chunk; atomic scatter only).  With the atomic scatter, device
 * buffers and a one-chunk interior pass, the point stage clears A and b beside its own
 * work (phase 0 is then only the reset of the status word; phases 1 and 3 include the
 * clear) and the boundary pass runs beside the interior kernels from the end of that
 * point stage; otherwise it runs beside them from the start.  Phase 2 is only the part of
 * the boundary pass that outlasts the interior kernels. */
double gales_asm_last_phase_ms(gales_asm* h, int32_t phase);
/* Number of kernel launches made by the library since the handle was created. */
int64_t gales_asm_launch_count(gales_asm* h);

/* GALES mesh files, replacing the reader of Mesh::mesh_reader (src/fem/mesh/mesh.hpp:
 * 147-456: read_header, read_elements, read_sides, read_nodes, el_side_info).  Text
 * lines "MESH! 2D|3D", "nodes N", "elements N", "sides N", one bounds line per
 * dimension, then N "Node gid x y [z] flag", N "Element gid pid nnodes n... flag" and
 * N "Side gid pid nsn n... flag" lines; tokens separated by spaces or commas.
 * pid >= 0 reads the elements and sides of that partition (as one MPI rank of the
 * reference does), pid < 0 all of them.  The nodes are the sorted distinct gids the
 * read elements use (local id = position).  A boundary element's local side gets the
 * flag of the Side line with the same nodes when all its nodes are boundary nodes;
 * sides with flag > 0 become gales_mesh_desc boundary sides.  Host-only, no GPU use.
 * On failure err (err_len bytes, may be NULL) holds the reason and the line. */
typedef struct gales_mesh_file gales_mesh_file;
int gales_mesh_read(const char* path, int32_t pid, gales_mesh_file** out, char* err, int32_t err_len);
/* Fills desc with pointers into the mesh file's arrays (valid until it is freed);
 * node_gid[n_nodes] and el_gid[n_elements] give the file's gids (either may be NULL). */
int gales_mesh_file_desc(const gales_mesh_file* m, gales_mesh_desc* desc, const int64_t** node_gid,
                         const int64_t** el_gid);
void gales_mesh_file_free(gales_mesh_file* m);

#ifdef __cplusplus
}
#endif

#endif /* GALES_ASM_H_ */
