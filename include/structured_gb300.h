/* structured_gb300 — C ABI of the GB300 residual / discrete-adjoint path.
 *
 * Drop-in for the hot path of anandpratap/structured.  The reference has no
 * FFI; its boundary is the templated C++ class interface bound at compile
 * time.  Each entry point below names the reference member it replaces.
 *
 * Conventions (all entry points):
 *   - return int status: ST_OK (0) or a negative ST_ERR_* code; the message
 *     of the last failure on the calling thread is st_last_error();
 *   - the caller owns host buffers, the context owns device buffers; the
 *     solver, adjoint, explicit-stage and MLP buffers are allocated on their
 *     first use and kept; no other call allocates (except where stated);
 *   - one context = one device + one CUDA stream; calls on one context are
 *     not thread safe;
 *   - state layout is the reference's q[i][j][k]: cells i in [0,nic),
 *     j in [0,njc), k in [0,nq), row-major FP64 (src/solver/solution.cpp:28),
 *     nic = ni-1, njc = nj-1; nq = 4 laminar, 5 with Spalart-Allmaras
 *     (k=4 holds rho*nu_tilde in the reference's ntrans slot,
 *     src/solver/solution.cpp:9,43-45).
 */
#ifndef STRUCTURED_GB300_H
#define STRUCTURED_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ST_OK = 0,
    ST_ERR_ARG = -1,          /* bad argument or size */
    ST_ERR_CUDA = -2,         /* CUDA runtime / launch failure */
    ST_ERR_NONFINITE = -3,    /* NaN/Inf detected in a result */
    ST_ERR_NOCONV = -4,       /* iterative solve did not converge */
    ST_ERR_TIMEOUT = -5,      /* bounded device wait expired (no current kernel waits on a flag) */
    ST_ERR_UNSUPPORTED = -6   /* option not built */
};

/* Boundary types, faces: src/model/bc.h:8-11 and src/model/bc.cpp:465-526. */
enum { ST_BC_FREESTREAM = 0, ST_BC_SLIPWALL = 1, ST_BC_WALL = 2, ST_BC_OUTFLOW = 3,
       ST_BC_PERIODIC = 4, ST_BC_ISOTHERMALWALL = 5, ST_BC_WAKE = 6 };
enum { ST_FACE_BOTTOM = 0, ST_FACE_RIGHT = 1, ST_FACE_TOP = 2, ST_FACE_LEFT = 3 };
enum { ST_VISC_POWER = 0, ST_VISC_SUTHERLAND = 1 };
enum { ST_TURB_NONE = 0, ST_TURB_SA = 1 };
/* [solver] flux: Roe (flux.cpp:51-146) or AUSM (flux.cpp:148-224, the reference's default) */
enum { ST_FLUX_ROE = 0, ST_FLUX_AUSM = 1 };

/* One [[boundary]] table.  start/end are ghost-padded indices along the face;
 * a negative end counts from the end as in BoundaryContainer::get_index
 * (src/model/bc.cpp:436-457). */
typedef struct st_bc {
    int32_t type, face, start, end;
    double u, v, T;
} st_bc;

/* Case setup: the [freestream], [solver], [source] keys of
 * src/utils/config.cpp:32-87 plus the keys this project adds. */
typedef struct st_case {
    int32_t ni, nj;                 /* vertices */
    int32_t order, lhs_order;       /* MUSCL order for the residual / Jacobian */
    int32_t viscosity_law;          /* ST_VISC_* */
    int32_t turbulence;             /* ST_TURB_* */
    int32_t nbc;
    int32_t plate_vertex;           /* first no-slip wall vertex (objective) */
    int32_t flux;                   /* ST_FLUX_*; the hand-written adjoint reverses both */
    double rho_inf, u_inf, v_inf, p_inf, T_inf, mu_inf, pr_inf;
    double dpdx, dpdy;              /* [source] body force */
    double nu_tilde_inf;            /* SA freestream nu_tilde */
    double plate_x_end;             /* objective integrates Cf dx for x <= this */
    const st_bc* bcs;
} st_case;

typedef struct st_ctx st_ctx;

typedef struct st_solve_stats {
    int32_t iterations;             /* Krylov iterations used */
    int32_t converged;              /* 1 if the relative tolerance was met */
    double residual0, residual;     /* initial / final linear residual 2-norms */
} st_solve_stats;

/* Pseudo-time Newton parameters: the [solver] keys of src/utils/config.cpp:
 * 42-56 (cfl, ramps, tolerance, iteration_max) plus the Krylov settings. */
typedef struct st_solve_params {
    int32_t max_steps;                    /* iteration_max */
    int32_t krylov_m;                     /* GMRES restart length */
    int32_t krylov_maxit;                 /* GMRES iterations per pseudo-time step */
    int32_t cfl_ramp, cfl_ramp_iteration;
    int32_t under_relaxation_ramp, under_relaxation_ramp_iteration;
    int32_t max_failures;                 /* divergence-guard restarts allowed */
    int32_t min_steps;                    /* Newton steps taken before the tolerance is checked */
    double cfl, cfl_max, cfl_ramp_exponent;
    double under_relaxation, under_relaxation_ramp_exponent;
    double tolerance;                     /* stop when max_k ||R_k||_2 <= tolerance */
    double rel_tolerance;                 /* ... or <= rel_tolerance * initial */
    double krylov_rtol;
    double ser_exponent;                  /* > 0: also CFL >= cfl (r0/r)^ser_exponent */
    double divergence_factor;             /* unused (kept for layout); see reject_factor */
    double cfl_growth;                    /* > 0: CFL *= cfl_growth after each accepted full step */
    double reject_factor;                 /* a step that raises max ||R|| by more than this is undone, CFL / 10 */
    double max_rel_drho;                  /* > 0: damp the update so |d rho / rho| <= this in every cell */
    double nut_floor;                     /* > 0, SA: rho nu_tilde keeps at least this fraction of its old
                                             value (0 = off: converged SA-neg states may hold nu_tilde < 0) */
    double cfl_min;                       /* lower bound for CFL cuts */
} st_solve_params;

const char* st_last_error(void);
int st_version(void);

/* Lifecycle: replaces Mesh::setup (src/utils/mesh.cpp:392-414) — metrics
 * (Mesh::calc_metrics, mesh.cpp:172-205), fluid model, boundary container and
 * solution arrays.  xv, yv: vertices [ni][nj] (Mesh::xv/yv).  device < 0
 * means the current device. */
int st_create(const st_case* c, const double* xv, const double* yv, int device, st_ctx** out);
int st_destroy(st_ctx* ctx);
int st_dims(const st_ctx* ctx, int* nic, int* njc, int* nq);

/* State transfer (Solution::q).  Host buffers [nic][njc][nq].  Synchronous;
 * the copies run on the context's copy stream after the work already queued. */
int st_set_state(st_ctx* ctx, const double* q_host);
int st_get_state(st_ctx* ctx, double* q_host);
/* SA production multiplier beta [nic][njc] (default 1). */
int st_set_beta(st_ctx* ctx, const double* beta_host);
int st_get_wall_distance(st_ctx* ctx, double* d_host);

/* Residual: EulerEquation::calc_residual(q, rhs, lhs)
 * (src/model/eulerequation.h:53, eulerequation.cpp:202-232), evaluated on the
 * context's state; lhs != 0 selects lhs_order.  rhs_host [nic][njc][nq] may be
 * NULL to keep the result on the device.  The copy to rhs_host overlaps the
 * last pass: the cell pass runs in up to 8 bands and each band goes out on
 * the copy stream while the next computes (page-locked rhs_host lets the
 * copies run asynchronously). */
int st_residual(st_ctx* ctx, int lhs, double* rhs_host);
/* Same on caller-provided device buffers (q_dev, rhs_dev: [nic][njc][nq]);
 * beta_dev may be NULL (beta = 1). */
int st_residual_device(st_ctx* ctx, const double* q_dev, const double* beta_dev,
                       double* rhs_dev, int lhs);

/* Which kernels evaluate the FP64 residual of st_residual*, the Newton and
 * explicit solvers: path 1 = tiled i- and j-sweeps whose CTAs stage their
 * tile of primitive records plus a two-cell halo in shared memory by TMA and
 * keep slopes and face fluxes on chip; path 0 (the default) = one pass per
 * stage (slopes, i-faces, j-faces, cells) through HBM, measured faster on
 * this FP64-issue-bound residual.
 * Both compute the stages of calc_residual (eulerequation.cpp:168-232) with
 * the same face arithmetic.  The network-beta residual and JVPs always use the
 * per-stage passes.  *active (may be NULL) = 1 if the tiled sweeps now run.
 * ST_ERR_UNSUPPORTED for path 1 when the driver offers no tensor-map encoder. */
int st_set_residual_path(st_ctx* ctx, int path, int* active);

/* Local time step: EulerEquation::calc_dt(cfl), eulerequation.cpp:237-259.
 * dt_host [nic][njc][nq] may be NULL. */
int st_dt(st_ctx* ctx, double cfl, double* dt_host);
/* L2 norm of each residual component of the last st_residual
 * (Solver::step, src/solver/solver.cpp:125-134); out[nq]. */
int st_norms(st_ctx* ctx, double* out);

/* Wall skin friction at the j=0 faces, the reference's
 * Cf = mu_inf (du/dy - dv/dx)/q_inf (IOManager::write_surface,
 * src/utils/io.cpp:217-226), of the current state; cf_host [nic] (may be
 * NULL).  J is sum Cf dx over plate faces with x <= plate_x_end, reduced on
 * the device (warp-shuffle tree, fixed order). */
int st_skin_friction(st_ctx* ctx, double* cf_host, double* J);
/* Same on the device without synchronising: cf_dev [nic] and J_dev [1]
 * (either may be NULL) are written on the context stream. */
int st_skin_friction_device(st_ctx* ctx, double* cf_dev, double* J_dev);
/* Velocity gradients (u_x, u_y, v_x, v_y) of the current state at the j = 0
 * faces, [nic][4] on the host: the row of the reference's grad_u_eta /
 * grad_v_eta that IOManager::write_surface reads for Cf and the viscous
 * Cl/Cd (src/utils/io.cpp:217-236).  The first call allocates a context
 * buffer of nic * 32 bytes. */
int st_wall_gradients(st_ctx* ctx, double* out_host);

/* Forward-mode Jacobian-vector product (dR/dQ) v + (dR/dbeta) vb on the
 * context state; vb may be NULL.  Replaces one column sweep of ADOL-C's
 * sparse_jac (src/solver/solver.cpp:156). */
int st_jvp_device(st_ctx* ctx, const double* v_dev, const double* vb_dev, double* jv_dev, int lhs);

/* Hand-written discrete adjoint: psi_q = (dR/dQ)^T psi, psi_b = (dR/dbeta)^T psi
 * on the context state (no tape, face fluxes recomputed).  Either output may
 * be NULL.  All device pointers. */
int st_vjp_device(st_ctx* ctx, const double* psi_dev, double* out_q_dev, double* out_beta_dev, int lhs);
/* Host-buffer variant.  psi goes in on the copy stream while the forward
 * passes run; out_beta goes out as soon as it is final; out_q follows the
 * last pass band by band.  Page-locked host buffers let the copies overlap
 * the passes. */
int st_vjp(st_ctx* ctx, const double* psi_host, double* out_q_host, double* out_beta_host, int lhs);
/* Residual and adjoint of the same state in one sweep (the forward passes
 * are shared and each face pass computes its flux and its reverse at once):
 * rhs as st_residual_device, products as st_vjp_device.  psi must not alias
 * rhs.  Device pointers; outputs may be NULL except rhs. */
int st_residual_vjp_device(st_ctx* ctx, const double* psi_dev, double* rhs_dev, double* out_q_dev,
                           double* out_beta_dev, int lhs);
/* Host-buffer variant of st_residual_vjp_device (on the context state), with
 * the copies overlapped as in st_vjp; rhs goes out while the gather runs. */
int st_residual_vjp(st_ctx* ctx, const double* psi_host, double* rhs_host, double* out_q_host,
                    double* out_beta_host, int lhs);
/* Kernel launches one st_residual_vjp_device call makes. */
int st_fused_launch_count(st_ctx* ctx, int lhs);

/* Block Jacobian dR/dQ of the residual (lhs != 0: lhs_order) at the context
 * state, 13-point stencil of nq x nq blocks, from exact forward-mode JVPs over
 * a 5x5 cell colouring.  Replaces ADOL-C's sparse_jac and the COO buffers of
 * src/solver/solver.cpp:156-171.  Ghosts that copy distant cells add blocks
 * outside that stencil: a bottom wake cut (bc.cpp:224-263) and periodic
 * boundaries in i (bc.cpp:329-365, the channel example).  Each copied ghost
 * couples four rows next to its boundary to the cell it copies; those partner
 * blocks are assembled too and used by every operator product and solve below,
 * but not by the preconditioner.  ST_ERR_UNSUPPORTED (this call, st_solve and
 * the adjoint and tangent solves) for a wake cut on another face or on a
 * corner ghost, periodic boundaries in j or not covering every row, both kinds
 * together, and grids one cell wide. */
int st_jacobian_assemble(st_ctx* ctx, int lhs);
/* Copy of the blocks, [nic][njc][13][nq][nq] (row component major); offsets
 * (di,dj): (0,0),(-1,0),(1,0),(0,-1),(0,1),(-2,0),(2,0),(0,-2),(0,2),
 * (-1,-1),(-1,1),(1,-1),(1,1).  With wake or periodic boundaries these are
 * the local part (the copied ghosts held fixed); the partner blocks are not
 * copied. */
int st_jacobian_blocks(st_ctx* ctx, double* blocks_host);
/* out = J v (transpose != 0: J^T v) with the assembled blocks. */
int st_jacobian_apply_device(st_ctx* ctx, const double* v_dev, double* out_dev, int transpose);
/* One linear solve of the implicit step, (I/dt(cfl) - J) x = b (or its
 * transpose): the set_lhs / set_rhs / solve of the reference's linear-solver
 * classes (src/linearsolver/ls_eigen.cpp:23-71), here restarted GMRES with a
 * block-tridiagonal j-line preconditioner; x holds the initial guess. */
int st_linear_solve_device(st_ctx* ctx, double cfl, const double* b_dev, double* x_dev, int transpose,
                           int krylov_m, int maxit, double rtol, st_solve_stats* stats);
/* Pseudo-time Newton to steady state on the context state: Solver::solve /
 * Solver::step (src/solver/solver.cpp:53-236) with the implicit (ADOL-C) path.
 * history (may be NULL) receives per step [step, cfl, krylov iterations,
 * ||R_0..nq-1||_2]; *steps_done the steps taken.  Returns ST_ERR_NOCONV if the
 * tolerance is not reached in max_steps. */
int st_solve(st_ctx* ctx, const st_solve_params* params, st_solve_stats* stats, double* history,
             int history_len, int* steps_done);
/* grad_dev = d(sum_i w_i Cf_i)/dQ at the context state for wall weights
 * w_host[nic] (drag: w = dx; inversion misfit: w = 2 (Cf - Cf*)). */
/* Explicit marching of Solver::step's explicit branch (src/solver/solver.cpp:
 * 103-116): scheme 0 = forward_euler (q += R dt), 1 = rk4_jameson (stages
 * q_s = q + R(q_{s-1}) dt / (4 - s), s = 0..3, q_{-1} = q), dt from calc_dt
 * at each step's start (every component; the reference leaves the transport
 * slot unset).  Norms of the last stage's residual, as the reference logs
 * them, every `check_every` steps into history ([step, norms...]); stops at
 * max_k ||R_k|| <= tolerance (0: run all steps; ST_ERR_NOCONV if a positive
 * tolerance is not reached).  Periodic and wake boundaries are supported. */
int st_explicit_solve(st_ctx* ctx, int scheme, double cfl, int steps, double tolerance, int check_every,
                      double* history, int history_len, int* steps_done);
int st_cf_gradient_device(st_ctx* ctx, const double* w_host, double* grad_dev);
/* Adjoint solve (dR/dQ)^T psi = b with the exact Jacobian of the residual;
 * the preconditioner adds I/dt(cfl_prec).  psi holds the initial guess. */
int st_adjoint_solve_device(st_ctx* ctx, const double* b_dev, double* psi_dev, double cfl_prec, int krylov_m,
                            int maxit, double rtol, st_solve_stats* stats);

/* Tangent (forward sensitivity) solve (dR/dQ) dq = b with the exact Jacobian,
 * the dual of st_adjoint_solve_device; used to cross-check adjoint gradients. */
int st_tangent_solve_device(st_ctx* ctx, const double* b_dev, double* dq_dev, double cfl_prec, int krylov_m,
                            int maxit, double rtol, st_solve_stats* stats);

/* State of the implicit solve's preconditioner after the last factorisation
 * (st_solve, st_linear_solve_device): strip_unknowns = unknowns of the wake
 * strip level (0: no wake cut, partner blocks folded into the ILU(0) pattern
 * instead, or more than 1024 unknowns, in which case only the block ILU(0)
 * runs); strip_active = 1 if the last forward factorisation built the strip's
 * inverse (0 after a transposed one, or when its dense block was singular);
 * strip_factorisations counts strip builds; strip_host_ms is the host time of
 * the last one (gather, dense inverse, upload).  Any pointer may be NULL.
 * No counterpart in the reference (its sparse LU needs no preconditioner). */
int st_precond_info(st_ctx* ctx, int* strip_unknowns, int* strip_active, int* strip_factorisations,
                    double* strip_host_ms);

/* Kernel launches one st_residual_device / st_vjp_device call makes. */
int st_launch_counts(st_ctx* ctx, int lhs, int* residual, int* vjp);

/* L2 norm of each of the nq components of a residual that is already on the
 * device (rhs_dev: [ncell][nq] doubles), written to out_dev[nq] on `stream`
 * (a cudaStream_t; NULL = default stream); asynchronous.  This entry point
 * has no counterpart in the reference.  It allocates no device memory, for
 * callers that cannot allocate once running (an application that has reserved
 * the device for its own pool, or a loop that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree): its partial sums live in a fixed
 * 64 KiB device array inside the library, held by every device that loads it
 * until the process exits.  Limit: nq <= 8.  Every call looks up that
 * array's address on the current device (cudaGetSymbolAddress, which
 * allocates nothing), so the address survives a device reset; the first call
 * on a device loads the library's device code there, so make it outside any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * race. */
int st_norms_noalloc(const double* rhs_dev, long long ncell, int nq, double* out_dev, void* stream);

/* ---- learned SA correction (no counterpart in the reference) -------------
 * A 4-64-64-1 MLP (tanh, tanh, softplus) maps four features of each cell to
 * the SA production multiplier beta: P/(P+D) with beta = 1, chi, log10 y+
 * (u_tau from the wall shear of the cell's column) and |S|/|Omega|.  Weights
 * are BF16, products run on the tensor cores with FP32 accumulation; the
 * FP32 master copy is trained by Adam.  Enabled, the residual kernels of
 * st_residual*, st_jvp_device and st_solve evaluate beta in-kernel from the
 * current state (Jacobian products hold it fixed); the fused
 * residual+adjoint pipeline keeps using the beta array. */
int st_mlp_param_count(void);                                /* FP32 master parameters */
int st_mlp_init(st_ctx* ctx, unsigned long long seed);       /* Xavier-uniform weights, zero biases */
int st_mlp_set_params(st_ctx* ctx, const float* params);    /* [st_mlp_param_count()] */
int st_mlp_get_params(st_ctx* ctx, float* params);
int st_mlp_set_normalization(st_ctx* ctx, const float mean[4], const float stdev[4]);
int st_mlp_enable(st_ctx* ctx, int on);
/* Adam (lr, beta1 0.9, beta2 0.999) on (1/batch) sum (beta - target)^2 over
 * batches drawn with replacement from n device samples (features [n][4],
 * raw; targets [n]); loss_host (optional) receives one loss per step. */
int st_mlp_train(st_ctx* ctx, const float* feat_dev, const float* target_dev, long n, int steps, int batch, float lr,
                 unsigned long long seed, float* loss_host);
/* Gradient of the training loss of one batch, without an update: the batch
 * st_mlp_train draws at its step `step` (0-based count of steps since
 * st_mlp_init) with this seed, the same forward and backward kernels and the
 * same fixed-order reduction, in the FP32 master layout
 * (grad_host[st_mlp_param_count()]); loss_host (optional) the batch loss. */
int st_mlp_grad(st_ctx* ctx, const float* feat_dev, const float* target_dev, long n, int batch,
                unsigned long long seed, int step, float* grad_host, float* loss_host);
int st_sa_features(st_ctx* ctx, float* feat_dev);           /* raw features of the state, [ncell][4] */
int st_mlp_beta(st_ctx* ctx, double* beta_dev);             /* network beta of the state, [ncell] */

/* Diagnostics: dense FP64 FMA throughput of this device (TFLOP/s). */
int st_probe_fp64(st_ctx* ctx, double* tflops);
/* Diagnostics: the kernels' Newton-Raphson reciprocal and square roots on a
 * device array x_dev[n] of positive normal doubles; out_dev[n][5] receives
 * 1/x, 1/sqrt(x), sqrt(x), and the (sqrt(x), 1/sqrt(x)) pair of the combined
 * routine, for tests against correctly rounded values.  Synchronises. */
int st_probe_nr_math(const double* x_dev, long long n, double* out_dev);
/* Runs one pipeline on the context state (which = 0: residual; 1: adjoint VJP
 * with psi = the context's last residual; 2: residual + VJP in one sweep) with a CUDA event after every
 * launch: ms[k] is the device time of launch k, names a comma-separated list
 * of kernel names, *n the launch count (at most max_n). */
int st_profile_pipeline(st_ctx* ctx, int which, int lhs, double* ms, int max_n, char* names, int names_len,
                        int* n);
/* Device time (ms) of the last residual / VJP launch sequence, CUDA events on
 * the context stream (waits for them).  The *_device entry points are
 * asynchronous on the context stream; the host-buffer ones synchronise. */
int st_last_kernel_ms(st_ctx* ctx, double* residual_ms, double* vjp_ms);
/* Pointer to the context's device state / stream (for zero-copy callers). */
int st_device_state(st_ctx* ctx, double** q_dev, double** rhs_dev, void** stream);

#ifdef __cplusplus
}
#endif
#endif
