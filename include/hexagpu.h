/*
 * hexagpu.h — C ABI of the GB300-native finite-element solve path of HEXA TopOpt.
 *
 * One shared library (libhexagpu.so) exports plain C entry points: no C++ or
 * torch types cross this boundary, every array is a plain pointer plus sizes.
 * Each array argument may be a HOST pointer (pageable or pinned) or a DEVICE
 * pointer on the context's GPU; the library detects which with
 * cudaPointerGetAttributes and copies only what lives on the host.
 *
 * Layouts follow the reference (v119_2025_12_19_HEXATOP_AWS):
 *   - structured grid of nx*ny*nz hex8 elements of size dx*dy*dz
 *     (src/Mesh/Mesh.jl:23-60): node (i,j,k), 0-based, has index
 *     n = i + (nx+1)*(j + (ny+1)*k); element (i,j,k) has index
 *     e = i + nx*(j + ny*k); element local nodes n1..n8 as Mesh.jl:45-53.
 *   - displacement / force vectors are interleaved xyz per node (AoS),
 *     dof = 3*n + c, length 3*nNodes (src/Solvers/GPUSolver.jl:100-108).
 *   - per-element modulus factor: the reference passes `E .* density`
 *     (GPUSolver.jl:254); SIMP callers pass Emin + rho^p (E0 - Emin).
 *
 * Status codes: 0 converged / ok, 1 not converged (best iterate returned,
 * as GPUSolver.jl:439-443), negative = error, message in hexa_last_error().
 * A context is not reentrant: use one per host thread (the reference's
 * workspaces are process globals, GPUSolver.jl:63).
 */
#ifndef HEXAGPU_H
#define HEXAGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HEXA_OK 0
#define HEXA_NOT_CONVERGED 1
#define HEXA_ERR_ARG (-1)
#define HEXA_ERR_CUDA (-2)
#define HEXA_ERR_NOMEM (-3)
#define HEXA_ERR_CORRUPT_INPUT (-4) /* NaN/Inf in the stiffness diagonal: GPUSolver.jl:310-315 */
#define HEXA_ERR_NO_DEVICE (-5)     /* "CUDA not functional!": GPUSolver.jl:470-472 */
#define HEXA_ERR_TOO_LARGE (-6)     /* grid beyond HEXA_NOALLOC_MAX_NODES (hexa_filter_noalloc) */

typedef struct hexa_ctx hexa_ctx;

typedef struct hexa_grid {
  int32_t nx, ny, nz; /* elements per axis (geometry.nElem_*_computed) */
  double dx, dy, dz;  /* element edge lengths (geometry.d*_computed) */
} hexa_grid;

/* Dirichlet set. clamp_faces bit f fixes all 3 DOFs of every node on face f
 * (0: x=0, 1: x=max, 2: y=0, 3: y=max, 4: z=0, 5: z=max).  fixed_dof, when
 * not NULL, is 3*nNodes bytes, nonzero = fixed (the reference's
 * bc_indicator > 0 test, GPUSolver.jl:170-180).  The two are OR-ed. */
typedef struct hexa_bc {
  uint32_t clamp_faces;
  const uint8_t* fixed_dof;
} hexa_bc;

enum { HEXA_PRECOND_JACOBI = 0, HEXA_PRECOND_MULTIGRID = 1 };
enum { HEXA_PREC_FP64 = 0, HEXA_PREC_MIXED = 1, HEXA_PREC_FP32 = 2 };
enum { HEXA_SMOOTH_JACOBI = 0, HEXA_SMOOTH_CHEBYSHEV = 1 };
enum { HEXA_PRECOND_USED_JACOBI = 0, HEXA_PRECOND_USED_MULTIGRID = 1 };

/* Solver parameters.  The first block mirrors configs/default.yaml
 * solver_parameters (lines 209-237) as read by GPUSolver.jl:215-218 and
 * Solver.jl:57-59; the second block is new (precision and multigrid). */
typedef struct hexa_solve_params {
  double nu;                  /* Poisson ratio (material.nu) */
  double tol;                 /* solver_parameters.tolerance */
  int32_t max_iter;           /* solver_parameters.max_iterations (per attempt) */
  int32_t precond;            /* solver_parameters.preconditioner */
  double shift_factor;        /* solver_parameters.diagonal_shift_factor */
  double stagnation_tol;      /* solver_parameters.stagnation_tolerance */
  int32_t max_shift_attempts; /* solver_parameters.max_shift_attempts */
  double shift_multiplier;    /* solver_parameters.shift_multiplier */
  int32_t check_cadence;      /* 1: test ||r|| every iteration; 10: at k=1 and k%10==0 (GPUSolver.jl:379) */
  int32_t diag_quirk;         /* 1: x-diagonal of K0 for all 3 components (GPUSolver.jl:137) */
  /* --- additions --- */
  int32_t precision;          /* HEXA_PREC_* */
  int32_t mg_levels;          /* 0: automatic */
  int32_t pre_smooth, post_smooth;
  int32_t smoother;           /* HEXA_SMOOTH_* */
  double jacobi_omega;
  int32_t cheb_ratio;         /* Chebyshev smoothing interval [lmax/cheb_ratio, lmax] of D^-1 A (10) */
  int32_t coarse_iters;       /* Jacobi-PCG iterations of the coarsest-level solve when that grid
                                 has more than 640 DOFs (smaller ones are solved exactly, by the
                                 dense inverse of their operator) */
  double inner_tol;           /* mixed: relative tolerance of each FP32 correction solve */
  int32_t max_outer;          /* mixed: maximum refinement steps */
  int32_t use_graphs;         /* capture PCG iterations / V-cycles in CUDA graphs */
  int32_t graph_iters;        /* iterations per graph launch (host reads status between launches) */
  int32_t true_residual;      /* 1: recompute ||f-(K+sI)u||/||f|| in FP64 and iterate until <= tol */
  int32_t divergence_check;   /* 1: stop when rel > 10 or (k > 500 and rel > 100 best), GPUSolver.jl:397 */
  int32_t autotune;           /* mixed + multigrid: pick levels and smoother degree by short trial solves,
                                 cached per grid in the context (0: use mg_levels / pre_smooth / post_smooth) */
  int32_t mg_cycle;           /* coarse-grid visits per level: 1 V-cycle (default), 2 W-cycle */
} hexa_solve_params;

typedef struct hexa_solve_stats {
  int32_t status;
  int32_t iterations;       /* PCG iterations (FP32 inner iterations for mixed) */
  int32_t outer_iterations; /* mixed: refinement steps */
  int32_t attempts;         /* shift attempts used */
  int32_t precond_used;     /* HEXA_PRECOND_USED_*: "GMG_GPU" / "Jacobi_GPU" (GPUSolver.jl:463) */
  int32_t mg_levels;
  int32_t smooth_steps;     /* smoothing steps per side of the V-cycle that was used */
  double relres;            /* recursive ||r||/||f_free|| as GPUSolver.jl:380-382 reports */
  double true_relres;       /* ||f - (K+sigma I) u|| / ||f|| recomputed in FP64 */
  double shift;             /* sigma = shift_factor * max(diag K_ff) (GPUSolver.jl:343) */
  double max_diag;
  double compliance;        /* f . u (src/Main.jl:453) */
  double setup_ms;          /* device time: upload + hierarchy setup */
  double solve_ms;          /* device time: iterations + true residual */
  double total_ms;          /* host wall time of the call */
  double fine_applies;      /* fine-grid operator applications (FP64 + FP32) */
  double fine_applies_fp64;
  double unshifted_relres;  /* ||f - K u|| / ||f|| recomputed in FP64 without the shift (the residual of
                               the unshifted system; equals true_relres when sigma = 0; multi-RHS: the
                               largest over the columns; batches: NaN when sigma > 0) */
} hexa_solve_stats;

typedef struct hexa_filter_stats {
  int32_t status;
  int32_t iterations;       /* GPUHelmholtz.jl:224 final_iter */
  double relres;            /* GPUHelmholtz.jl:247 final_rel_res */
  double solve_ms;
} hexa_filter_stats;

/* ---- context ----------------------------------------------------------- */
/* A context replaces the reference's module-global workspaces
 * (GPUSolver.jl:63, GPUGeometricMultigrid.jl:37) and its CUDA.functional()
 * check (GPUSolver.jl:470-472: HEXA_ERR_NO_DEVICE); hexa_default_params gives
 * the configs/default.yaml solver_parameters defaults. */
int hexa_create(int32_t device, hexa_ctx** out);
void hexa_destroy(hexa_ctx* ctx);
const char* hexa_last_error(const hexa_ctx* ctx);
int hexa_version(void);
void hexa_default_params(hexa_solve_params* p);
/* device time of the last hexa_* call's timed region, ms (CUDA events) */
double hexa_last_device_ms(const hexa_ctx* ctx);
/* number of this library's kernels launched since the context was created */
int64_t hexa_kernel_launches(const hexa_ctx* ctx);

/* ---- element matrices (host) ------------------------------------------- */
/* Element.get_canonical_stiffness (src/Core/Element.jl:104-111), E = 1,
 * 24x24 column-major, DOF order node-major xyz over n1..n8.  Built in FP64
 * (the reference builds it in Float32 and promotes, GPUSolver.jl:248-249). */
int hexa_canonical_stiffness(double dx, double dy, double dz, double nu, double* ke_out);
/* Element.get_scalar_canonical_matrices (src/Core/Element.jl:113-134):
 * 8x8 Laplacian Ke and consistent mass Me.  quirk=1 keeps the reference's
 * top-face z = +dz (Element.jl:116); quirk=0 uses the true brick. */
int hexa_scalar_canonical_matrices(double dx, double dy, double dz, int32_t quirk,
                                   double* ke_out, double* me_out);

/* ---- (a) operator ------------------------------------------------------ */
/* y = (K(factor) + sigma I) x restricted to free DOFs, y = 0 at fixed DOFs;
 * the deterministic node-centric replacement of apply_A!
 * (GPUSolver.jl:322-330, matvec_unstructured_atomic_kernel! :91-128).
 * Entries of x at fixed DOFs are ignored (expand_kernel! semantics). */
int hexa_apply_operator(hexa_ctx* ctx, const hexa_grid* g, const hexa_bc* bc, double nu,
                        const double* factor, const double* x, double sigma, double* y);
/* The same operator in FP32 (the reference runs T = Float32 on its RTX profile, GPUSolver.jl:188-189). */
int hexa_apply_operator_f32(hexa_ctx* ctx, const hexa_grid* g, const hexa_bc* bc, double nu,
                            const float* factor, const float* x, float sigma, float* y);
/* No counterpart in the reference (a benchmark hook).
 * Times `reps` back-to-back launches of the operator kernel alone on the
 * context's stream with CUDA events (inputs already on the device) and
 * returns the mean launch duration in ms.  precision: HEXA_PREC_FP64 or
 * HEXA_PREC_FP32 (factor/x/y then float).  mode: 0 y = Ax, 1 y = Ax with
 * x.Ax, 2 y = b - Ax, 4 y = x + omega (b - Ax)/diag (damped Jacobi), 5 one
 * Chebyshev step written over its previous iterate (y). */
int hexa_time_operator(hexa_ctx* ctx, const hexa_grid* g, const hexa_bc* bc, double nu, int32_t precision,
                       int32_t mode, const void* factor, const void* x, const void* b, void* y, int32_t reps,
                       double* avg_ms);
/* diag(K_ff) per DOF (zero at fixed DOFs): compute_diagonal_atomic_kernel!
 * (GPUSolver.jl:130-144); diag_quirk as in hexa_solve_params. */
int hexa_operator_diagonal(hexa_ctx* ctx, const hexa_grid* g, const hexa_bc* bc, double nu,
                           const double* factor, int32_t diag_quirk, double* diag_out);

/* ---- (a)-(c) solve ------------------------------------------------------ */
/* Replaces GPUSolver.solve_system_gpu / gpu_matrix_free_cg_solve
 * (GPUSolver.jl:182-477): solves (K_ff + sigma I) u = f_free.
 * factor: nElem modulus factors; f: 3*nNodes forces (entries at fixed DOFs
 * ignored, as f[free_dofs] at GPUSolver.jl:292); u_guess may be NULL;
 * u_out: 3*nNodes, zeros at fixed DOFs (GPUSolver.jl:446-448). */
int hexa_solve(hexa_ctx* ctx, const hexa_grid* g, const hexa_bc* bc, const double* factor,
               const double* f, const hexa_solve_params* p, const double* u_guess,
               double* u_out, hexa_solve_stats* stats);

/* Same call with the reference's own argument types (GPUSolver.jl:467-469):
 * Float32 E, density (nElem), f (3*nNodes) and bc_indicator as the Julia
 * Matrix{Float32}(nNodes,3) in column-major order (>0 = fixed).  The factor
 * is Float64(Float32(E*density)) as GPUSolver.jl:254.  method_out receives
 * "GMG_GPU", "Jacobi_GPU" or "Failed_Corrupt_Input". */
int hexa_solve_system_gpu(hexa_ctx* ctx, const hexa_grid* g, float E, const float* bc_indicator,
                          const float* f, const float* density, const hexa_solve_params* p,
                          const float* u_guess, double* u_out, double* relres_out,
                          char* method_out, int32_t method_cap, hexa_solve_stats* stats);

/* Replaces Solver.solve_system for the gpu solver type (src/Solvers/Solver.jl:39-160),
 * the call the SIMP loop makes (src/Main.jl:439-443), with the same argument
 * types as hexa_solve_system_gpu plus the dispatcher's own:
 * min_stiffness_threshold, prune_voids and config["current_outer_iter"].  When
 * prune_voids is set, current_outer_iter >= 3 and fewer than 99 % of the
 * elements have density > min_stiffness_threshold * 1.01f (Solver.jl:66-90),
 * the system solved is the pruned one of MeshPruner.prune_system
 * (src/Mesh/MeshPruner.jl:10-87): those elements removed, the nodes no kept
 * element touches removed (their loads dropped), the shift taken from the
 * pruned diagonal; u_out then holds zeros at removed nodes, as
 * reconstruct_full_solution (MeshPruner.jl:89-107) writes.  On the structured
 * grid this is the full grid with the removed elements' factors set to zero
 * and the removed nodes' DOFs fixed.  No element kept: HEXA_ERR_ARG with the
 * reference's message.  active_elements (nullable) receives the number of
 * elements in the solved system.  u_prev may be NULL. */
int hexa_solve_system(hexa_ctx* ctx, const hexa_grid* g, float E, const float* bc_indicator, const float* f,
                      const float* density, float min_stiffness_threshold, int32_t prune_voids,
                      int32_t current_outer_iter, const hexa_solve_params* p, const float* u_prev, double* u_out,
                      double* relres_out, char* method_out, int32_t method_cap, hexa_solve_stats* stats,
                      int64_t* active_elements);

/* No counterpart in the reference (it solves one load case per call,
 * GPUSolver.jl:467-477): k load cases as one block PCG (each K0/factor load
 * serves k right-hand sides).  F and U are k consecutive 3*nNodes vectors. */
int hexa_solve_multi_rhs(hexa_ctx* ctx, const hexa_grid* g, const hexa_bc* bc, const double* factor,
                         int32_t k, const double* F, const hexa_solve_params* p, double* U,
                         hexa_solve_stats* stats);

/* No counterpart in the reference: `count` independent problems on grids of
 * uneven sizes solved together: one launch per kernel over all instances,
 * per-instance reductions and convergence, the PCG iteration and V-cycle
 * replayed from one CUDA graph.  grids[i], bcs[i] (clamp faces only:
 * fixed_dof must be NULL; bcs may be NULL for no clamps), factors[i] (nElem_i),
 * forces[i] (3*nNodes_i) and u_out[i] are per instance, host or device
 * pointers; all instances share the element size and nu.  Mixed precision
 * with the multigrid preconditioner only (FP32 GMG-PCG, FP64 reliable
 * updates to p->tol per instance); p->autotune picks the operator's z-brick
 * depth by timing.  Each instance's hierarchy halves every axis (an odd axis
 * rounded up, unless that axis' high face is clamped; no axis below 2
 * elements) down to at most 1000 nodes, or to at most p->mg_levels levels
 * when that is > 0; stats[i].mg_levels reports the count.  stats (nullable) receives count entries; the return is
 * HEXA_OK when every instance converged, HEXA_NOT_CONVERGED otherwise. */
int hexa_solve_batch(hexa_ctx* ctx, int32_t count, const hexa_grid* grids, const hexa_bc* bcs, double nu,
                     const double* const* factors, const double* const* forces, const hexa_solve_params* p,
                     double* const* u_out, hexa_solve_stats* stats);

/* ---- (d) Helmholtz density filter -------------------------------------- */
/* Replaces GPUHelmholtz.apply_gpu_filter! (GPUHelmholtz.jl:422-443):
 * solves (R^2 K_s + M_s) psi = sum_e rho_e vol/8 with Jacobi-PCG (at most
 * max_iter iterations, ||r||/||b|| checked every 10), returns the element
 * mean of psi.  precision: HEXA_PREC_FP64 or HEXA_PREC_FP32 (reference). */
int hexa_filter(hexa_ctx* ctx, const hexa_grid* g, const double* rho_in, double radius, double tol,
                int32_t max_iter, int32_t quirk, int32_t precision, double* rho_out,
                hexa_filter_stats* stats);

/* The filter of hexa_filter without any device allocation (this entry point
 * has no counterpart in the reference).  For callers that cannot allocate
 * device memory where they filter -- code running on its own stream while
 * another stream of its application is being captured into a CUDA graph, or
 * hosts whose own pool owns the device-memory budget.  All scratch lives in
 * one fixed device array inside the library (about 15 MB, held by every GPU
 * that loads the library until exit), so the grid may have at most
 * HEXA_NOALLOC_MAX_NODES nodes; larger grids return HEXA_ERR_TOO_LARGE.
 * rho_in and rho_out must be device pointers on the current device (host
 * arrays would need a staging allocation, and another GPU's arrays are not
 * this device's: HEXA_ERR_ARG); FP64 arithmetic, same algorithm and results
 * as hexa_filter with HEXA_PREC_FP64 (a NaN residual or a p.Ap breakdown
 * gives a NaN field).  The call synchronizes its stream and cannot itself be
 * captured: a stream that is capturing is refused (HEXA_ERR_ARG).  While the
 * application captures another stream, pass a non-blocking stream
 * (cudaStreamNonBlocking); NULL is the legacy default stream, whose work
 * joins a capture on any blocking stream.  The call returns when its work is
 * done, with the calling thread's capture mode as it found it.  Every call
 * reuses the array: calls that overlap on the GPU race and must be
 * serialised by the caller.  The first call on a device resolves the array's
 * device address; make it before any stream capture begins. */
#define HEXA_NOALLOC_MAX_NODES 262144
int hexa_filter_noalloc(const hexa_grid* g, const double* rho_in, double radius, double tol, int32_t max_iter,
                        int32_t quirk, double* rho_out, void* stream, hexa_filter_stats* stats);

/* The filter of hexa_filter over `count` grids of uneven sizes in one batch
 * (no counterpart in the reference): every Jacobi-PCG kernel is one launch
 * over all instances, each with its own dots, every-10 test and cap.  All
 * grids share the element size; rho_in[i]/rho_out[i] host or device. */
int hexa_filter_batch(hexa_ctx* ctx, int32_t count, const hexa_grid* grids, const double* const* rho_in,
                      double radius, double tol, int32_t max_iter, int32_t quirk, int32_t precision,
                      double* const* rho_out, hexa_filter_stats* stats);

/* ---- (f) stress post-processing ---------------------------------------- */
/* Replaces Stress.compute_stress_field (src/Core/Stress.jl:286-339, kernel
 * :159-285): per element at its centre the stress of E_loc = E * density,
 * the principal stresses (descending) with the directions of the largest and
 * smallest, von Mises, the L1 norm of the principal stresses and, when voigt
 * is not NULL, the Voigt stress (xx, yy, zz, xy, yz, xz).  u is the FP64
 * solution (3*nNodes), rounded to Float32 as the reference does; outputs are
 * Float32, element-major (principal[3e+i], voigt[6e+i], dir_*[3e+i]);
 * elements with density < 1e-6 get zeros.  Arrays host or device. */
int hexa_stress_field(hexa_ctx* ctx, const hexa_grid* g, const double* u, const float* density, float E, float nu,
                      float* principal, float* vonmises, float* voigt, float* l1, float* dir_max, float* dir_min);

/* Replaces the field mapping of MeshRefiner.refine_mesh_and_fields
 * (src/Mesh/MeshRefiner.jl:188-240): the old cell-centred density (old grid
 * old_g, element order x fastest) interpolated trilinearly at the centroids
 * of the new grid new_g spanning the same box (lengths lx, ly, lz), projected
 * (> 0.4 -> 1, < 0.2 -> 1e-4) when projection is 1 ("hard" update); alpha
 * (nullable) is carried by nearest lower-corner cell into new_alpha
 * (nullable).  Float32 throughout; arrays host or device. */
int hexa_remap_fields(hexa_ctx* ctx, const hexa_grid* old_g, const hexa_grid* new_g, double lx, double ly, double lz,
                      const float* density, const float* alpha, int32_t projection, float* new_density,
                      float* new_alpha);

/* Warm start across a refinement: the nodal displacement field u_old
 * (3 per node, node-major xyz, grid old_g) interpolated trilinearly onto the
 * nodes of new_g spanning the same box, in FP64.  The reference resets U to
 * zero after MeshRefiner grows the grid (src/Main.jl:412-413); passing u_new
 * as the next solve's u_guess changes only where that solve starts.  Arrays
 * host or device. */
int hexa_remap_displacement(hexa_ctx* ctx, const hexa_grid* old_g, const hexa_grid* new_g, const double* u_old,
                            double* u_new);

/* ---- density update between solves (TopOpt.jl:211-482) ---------------- */
/* The scalars update_density! reads from its arguments and its config;
 * defaults are the reference's get(...) defaults. */
typedef struct hexa_density_update_params {
  float E;                                 /* Young's modulus (argument E) */
  float l1_stress_allowable;               /* argument l1_stress_allowable */
  int32_t iter;                            /* argument iter */
  int32_t number_of_iterations;            /* argument number_of_iterations */
  float min_density;                       /* argument min_density (1e-3) */
  float max_density;                       /* argument max_density (1.0) */
  float max_domain_dim;                    /* geometry.max_domain_dim (Float32) */
  float filter_R_init_perc;                /* optimization_parameters..., 0 */
  float filter_R_interm_perc;              /* 0 */
  float filter_R_final_perc;               /* 0 */
  float filter_R_interm_iter_perc;         /* 50 */
  float minimum_filter_radius_as_elements; /* 2.5 */
  float filter_tolerance;                  /* solver_parameters.filter_tolerance, 1e-5 */
  float final_density_threshold;           /* 0.95 */
  float max_culling_ratio;                 /* 0.1 */
  int32_t hard_update;                     /* density_update_method == "hard" (default "soft") */
  int32_t filter_max_iter;                 /* 200, as apply_gpu_filter! */
  int32_t filter_precision;                /* HEXA_PREC_FP32 (the reference's Float32 filter) or FP64 */
} hexa_density_update_params;

/* update_density!'s return tuple (mean_change, R_length, current_threshold,
 * filter_time, filter_iters, filter_res) and the counts behind it. */
typedef struct hexa_density_update_stats {
  int32_t status;              /* 0 updated; 1 skipped: NaN in the stress field (TopOpt.jl:230-236) */
  int32_t filter_used;         /* R_effective > 1e-4 */
  int32_t filter_nan_fallback; /* the filtered field held a NaN: the proposal was used (TopOpt.jl:360-363) */
  int32_t filter_iters;
  float mean_change;
  float R_length;
  float current_threshold;
  float R_effective;           /* R_length / 2.5, the radius given to the filter */
  double filter_time;          /* seconds of filter PCG (device time) */
  double filter_res;
  int64_t active_count;        /* after the clamp; protected elements by their original density */
  int64_t candidates;          /* unprotected elements with min_density < rho < current_threshold */
  int64_t culled;              /* candidates set to min_density */
} hexa_density_update_stats;

void hexa_default_density_update_params(hexa_density_update_params* p);

/* Replaces TopologyOptimization.update_density!(density, l1_stress_norm_field,
 * protected_elements_mask, E, l1_stress_allowable, iter,
 * number_of_iterations, original_density, min_density, max_density, config,
 * elements) (src/Optimization/TopOpt.jl:211-482) on the structured grid g:
 * density (Float32, in/out) is updated in place, the filter is this
 * library's (the GPU path of TopOpt.jl:310-327).  protected_mask (one byte
 * per element, nonzero = protected) may be NULL (none protected); arrays host
 * or device; at most 2^32 - 1 elements (HEXA_ERR_TOO_LARGE beyond). */
int hexa_update_density(hexa_ctx* ctx, const hexa_grid* g, float* density, const float* l1_stress,
                        const uint8_t* protected_mask, const float* original_density,
                        const hexa_density_update_params* p, hexa_density_update_stats* stats);

/* ---- (e) SIMP sensitivities and OC update ------------------------------ */
/* No counterpart in the reference (its update is the stress-ratio rule of
 * TopOpt.jl:211-482, hexa_update_density): the published SIMP/OC method
 * (modified SIMP modulus, OC with move limit and a bisection on the
 * Lagrange multiplier), reaching the same solve with SIMP factors. */
/* dc_e = -penal * rho_e^(penal-1) * (E0 - Emin) * u_e^T K0 u_e and
 * compliance = sum_e (Emin + rho_e^penal (E0-Emin)) u_e^T K0 u_e. */
int hexa_sensitivities(hexa_ctx* ctx, const hexa_grid* g, double nu, const double* rho,
                       const double* u, double Emin, double E0, double penal, double* dc_out,
                       double* compliance_out);
/* SIMP modulus factors Emin + rho^penal (E0-Emin) */
int hexa_simp_factors(hexa_ctx* ctx, int64_t n, const double* rho, double Emin, double E0,
                      double penal, double* factor_out);
/* Optimality-criteria update with a bisection on the Lagrange multiplier
 * until mean(x_new) = volfrac: x_new = clamp(x*sqrt(-dc/(lambda*dv)),
 * max(0,x-move), min(1,x+move)). */
int hexa_oc_update(hexa_ctx* ctx, int64_t n, const double* x, const double* dc, const double* dv,
                   double volfrac, double move, double* x_out, double* lambda_out);

#ifdef __cplusplus
}
#endif
#endif /* HEXAGPU_H */
