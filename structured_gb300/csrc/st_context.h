// Host-side context shared by the C-ABI translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/structured_gb300.h"
#include "st_common.cuh"

struct st_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    st_case c{};
    std::vector<st_bc> bcs;
    st::DevCase dc{};
    int nq = 4;
    size_t ncell = 0, npad = 0, nfi = 0, nfj = 0;

    // host copies
    std::vector<double> xv, yv, vol, nchi, neta, ds_min, wall_dx;

    // device buffers (double path)
    double *q = nullptr, *rhs = nullptr, *beta = nullptr, *P = nullptr;
    double *lim = nullptr, *Fi = nullptr, *Fj = nullptr, *Gi = nullptr, *Gj = nullptr;
    double *vol_d = nullptr, *ivol_d = nullptr, *geo_i = nullptr, *geo_j = nullptr, *wd = nullptr;
    double *nchi_d = nullptr, *neta_d = nullptr, *dsmin_d = nullptr, *dt = nullptr;
    double *norm_part = nullptr, *norm_out = nullptr, *cf = nullptr, *wall_dx_d = nullptr;
    st::DevBC* bcs_d = nullptr;
    int* err_d = nullptr;

    // forward-mode (dual) buffers, allocated on the first JVP call
    st::dual *qd = nullptr, *Pd = nullptr, *limd = nullptr;
    st::dual *Fdi = nullptr, *Fdj = nullptr, *Gdi = nullptr, *Gdj = nullptr, *rhsd = nullptr, *betad = nullptr;

    // adjoint buffers, allocated on the first VJP call
    double *Pbar = nullptr, *srec = nullptr, *arec_i = nullptr, *arec_j = nullptr;
    // implicit solver (allocated on first use)
    double *jac = nullptr, *jac1 = nullptr, *kv = nullptr, *kz = nullptr, *kw = nullptr, *kr = nullptr;
    double *kh = nullptr, *kpart = nullptr, *dq = nullptr, *qsave = nullptr;
    double* kzb = nullptr;   // flexible GMRES: preconditioned basis Z = M^{-1} V
    double* qtmp = nullptr;  // explicit RK stage state (Solution::q_tmp)
    double* wallg = nullptr; // wall-face velocity gradients [nic][4] (st_wall_gradients)
    float* lfac = nullptr;   // block ILU(0) factors, FP32: [cell][9][nq][nq]
    // non-local boundary copies (wake cut, periodic in i), per family: which
    // ghosts are copies, and the partner blocks that coupling adds to the
    // Jacobian, [line length][4][nq][nq] (st_partner.cuh)
    std::vector<int> pmask[3];
    int* pmask_d[3] = {nullptr, nullptr, nullptr};
    double* wpart[3] = {nullptr, nullptr, nullptr};
    // first-order partner blocks for the preconditioner when some partners lie
    // in the ILU(0) pattern (pfold) and the operator is second order
    double* wpart1[3] = {nullptr, nullptr, nullptr};
    bool partners_checked = false, has_partners = false, pfold = false;
    // wake strip preconditioner level (st_partner.cuh): strip cells, their
    // gathered blocks and time steps, the inverse of the strip block, a
    // residual buffer; strip_W1 the first-order wake partners it uses
    std::vector<int> strip_cells;
    int strip_ns = 0;
    int* strip_cells_d = nullptr;
    double *strip_jac_d = nullptr, *strip_dt_d = nullptr, *strip_inv_d = nullptr, *strip_res_d = nullptr;
    const double* strip_W1 = nullptr;
    bool strip_ready = false;
    double strip_host_ms = 0.0;   // host time of the last strip factorisation
    int strip_factored = 0;       // strip factorisations since the context was made
    bool pfam_on[3] = {false, false, false};
    // learned SA correction: BF16 weights, FP32 biases + normalisation, FP32
    // master parameters with Adam moments, training partials
    void* mlp_wb = nullptr;
    float *mlp_wf = nullptr, *mlp_master = nullptr, *mlp_loss = nullptr, *mlp_part = nullptr;
    size_t mlp_part_n = 0;
    int mlp_t = 0;
    int kv_m = 0;
    bool jac1_is_jac = false;
    double *psi_tmp = nullptr, *outq_tmp = nullptr, *outb_tmp = nullptr, *tape = nullptr;

    // tiled residual sweeps (st_tile.cuh): TMA descriptors of the primitive
    // array P for the i- and j-sweep boxes; res_path 1 = tiled sweeps (when
    // tile_ok), 0 = per-stage passes (the default: measured 4 % faster at
    // 4097x2049)
    CUtensorMap tmap_i{}, tmap_j{};
    bool tile_ok = false;
    int res_path = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // host-buffer entry points (st_residual, st_vjp, st_residual_vjp): the
    // host<->device copies run on their own stream so that they overlap the
    // pipeline (the host link moves about 0.2 TB/s each way).  hio is set
    // only during such a call.  The pipeline waits on hio.psi_ready before
    // its first read of psi; it queues the copy of each output to its host
    // destination as soon as the output is final; and its last per-cell pass
    // (k_cell; the gather with k_prim_adj behind it) runs in bands, each
    // band's output copied while the next band computes.
    struct HostIO {
        cudaEvent_t psi_ready = nullptr;
        double *rhs = nullptr, *outq = nullptr, *outb = nullptr;
    } hio;
    cudaStream_t xfer = nullptr;
    cudaEvent_t xev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // the host-buffer VJP's boundary ring of the state product (the two
    // outermost rows and columns, which the boundary reverse changes after
    // the gather), packed on the device and copied to page-locked host
    // memory; ring_pending: the call still has to scatter it into place
    double *ring_dev = nullptr, *ring_host = nullptr;
    bool ring_pending = false;
    static constexpr int kBands = 8;
    cudaEvent_t band_ev[kBands] = {};
    // per-launch profiling (st_profile_pipeline): an event after each launch
    bool prof_on = false;
    int prof_n = 0;
    cudaEvent_t prof_ev[33] = {};
    const char* prof_name[33] = {};
    float last_res_ms = 0.f, last_vjp_ms = 0.f;
    bool have_residual = false;
    bool res_pending = false, vjp_pending = false;
};

namespace stx {
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);
#define ST_CUDA(call)                                                  \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return stx::cuda_fail(e_, #call);       \
    } while (0)
#define ST_LAUNCH_CHECK(where)                                         \
    do {                                                               \
        cudaError_t e_ = cudaGetLastError();                           \
        if (e_ != cudaSuccess) return stx::cuda_fail(e_, where);       \
    } while (0)
inline unsigned grid_for(size_t n, unsigned threads = 256) {
    size_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > (1u << 30)) g = 1u << 30;
    return (unsigned)g;
}
// records a profiling event after a launch when profiling is on
inline void mark(st_ctx* x, const char* name) {
    if (!x->prof_on || x->prof_n >= 32) return;
    cudaEventRecord(x->prof_ev[x->prof_n + 1], x->stream);
    x->prof_name[x->prof_n + 1] = name;
    x->prof_n++;
}
// forward pipeline on (q -> rhs) for the double path; beta may be null.  Runs
// the tiled sweeps when selected and possible; run_residual_faces always runs
// the per-face passes, which also leave the face fluxes and gradient parts in
// Fi/Fj/Gi/Gj for callers that read them.
int run_residual(st_ctx* ctx, const double* q, const double* beta, double* rhs, int order);
// Queues the copy of `bytes` from device src to host dst on the copy stream,
// after the work queued so far on the context stream (ev: a free event).
inline int copy_out(st_ctx* x, cudaEvent_t ev, double* dst, const double* src, size_t bytes) {
    ST_CUDA(cudaEventRecord(ev, x->stream));
    ST_CUDA(cudaStreamWaitEvent(x->xfer, ev, 0));
    ST_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, x->xfer));
    return ST_OK;
}
// Synchronous copy between host memory and the context's device buffers: on
// the copy stream, after the work queued so far on the context stream.  Bulk
// host copies stay off the context stream: after one there, the next
// host-buffer call's copy of psi was measured not to overlap the forward
// passes (1.6 ms more per call at 4097x2049).
inline int copy_sync(st_ctx* x, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    ST_CUDA(cudaEventRecord(x->xev[0], x->stream));
    ST_CUDA(cudaStreamWaitEvent(x->xfer, x->xev[0], 0));
    ST_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, x->xfer));
    ST_CUDA(cudaStreamSynchronize(x->xfer));
    return ST_OK;
}
// Runs a per-cell pass launch(first, last) over the cells [0, ncell); with a
// host destination (dst non-null) in up to kBands bands, each band's nq
// doubles per cell copied from dev to dst while the next band computes.
template <class F>
int run_banded(st_ctx* x, double* dst, const double* dev, int nq, F&& launch) {
    const size_t n = x->ncell;
    const int nb = dst ? (int)std::min<size_t>(st_ctx::kBands, (n + 65535) / 65536) : 1;
    for (int b = 0; b < nb; b++) {
        const size_t f = n * b / nb, l = n * (b + 1) / nb;
        launch(f, l);
        if (dst) {
            int rc = copy_out(x, x->band_ev[b], dst + f * nq, dev + f * nq, (l - f) * nq * 8);
            if (rc) return rc;
        }
    }
    return ST_OK;
}
int run_residual_faces(st_ctx* ctx, const double* q, const double* beta, double* rhs, int order);
// forward-mode JVP of the order-`order` residual at the context state (async);
// freeze_nonlocal holds the periodic and wake ghosts' tangents at zero (the
// Jacobian's local part)
int run_jvp(st_ctx* ctx, const double* v_dev, const double* vb_dev, double* jv_dev, int order,
            int freeze_nonlocal = 0);
// time step into ctx->dt (async)
int run_dt(st_ctx* ctx, double cfl);
// L2 norms of rhs into host out[nq] (synchronises)
int run_norms(st_ctx* ctx, const double* rhs, double* out);
int ensure_adjoint_buffers(st_ctx* ctx);
}  // namespace stx
