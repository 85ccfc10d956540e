// C ABI of the hand-written discrete adjoint: launch sequence of the reverse
// passes in st_adjoint.cuh.
#include <algorithm>
#include <cstring>

#include "st_adjoint.cuh"
#include "st_context.h"

using namespace st;
using stx::fail;
using stx::grid_for;

namespace {

template <class T>
int alloc_d(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return stx::cuda_fail(e, "cudaMalloc (adjoint buffers)");
    return ST_OK;
}

// Grids whose host-buffer VJP runs the gather in bands with the boundary ring
// after it: at least eight bands' worth of cells and eight cells a side.
bool ringed_grid(const st_ctx* x) { return x->c.ni - 1 >= 8 && x->c.nj - 1 >= 8 && x->ncell >= 2 * 65536; }

int ensure(st_ctx* x) {
    if (x->Pbar) return ST_OK;
    const int nq = x->nq;
    const size_t ring = 2 * (size_t)(x->c.ni + 1) + 2 * (size_t)(x->c.nj - 1);
    int rc = ST_OK;
    if (rc == ST_OK) rc = alloc_d(&x->Pbar, x->npad * NP);
    if (rc == ST_OK) rc = alloc_d(&x->srec, x->ncell * SRW);
    if (rc == ST_OK) rc = alloc_d(&x->arec_i, x->nfi * ARW);
    if (rc == ST_OK) rc = alloc_d(&x->arec_j, x->nfj * ARW);
    if (rc == ST_OK) rc = alloc_d(&x->tape, std::max(1, x->c.nbc) * ring * RW);
    if (rc == ST_OK) rc = alloc_d(&x->psi_tmp, x->ncell * nq);
    if (rc == ST_OK) rc = alloc_d(&x->outq_tmp, x->ncell * nq);
    if (rc == ST_OK) rc = alloc_d(&x->outb_tmp, x->ncell);
    if (rc == ST_OK && ringed_grid(x)) {
        const size_t nr = ring_cells(x->c.ni - 1, x->c.nj - 1) * nq;
        rc = alloc_d(&x->ring_dev, nr);
        if (rc == ST_OK) {
            const cudaError_t e = cudaHostAlloc((void**)&x->ring_host, nr * sizeof(double), cudaHostAllocDefault);
            if (e != cudaSuccess) rc = stx::cuda_fail(e, "cudaHostAlloc (boundary ring)");
        }
    }
    if (rc) return rc;
    ST_CUDA(cudaMemsetAsync(x->srec, 0, x->ncell * SRW * 8, x->stream));
    return ST_OK;
}

// Residual (when rhs != null) and adjoint in one sweep: the forward passes are
// shared, and each face pass computes its flux and runs its reverse at once.
template <int NQ, int ORDER, int FLUX>
int launch_fused(st_ctx* x, const double* psi, double* rhs, double* outq, double* outb) {
    cudaStream_t s = x->stream;
    const DevCase& dc = x->dc;
    const unsigned gc = grid_for(x->ncell);
    k_prim<double, NQ><<<gc, 256, 0, s>>>(dc, x->q, x->P);
    stx::mark(x, "k_prim");
    {  // boundary pass with the ghost ring recorded before each BC, as grid-wide launches
        const unsigned gr = (unsigned)((2 * (x->c.ni + 1) + 2 * (x->c.nj - 1) + 255) / 256);
        const unsigned gb = (unsigned)((std::max(x->c.ni, x->c.nj) + 1 + 255) / 256);
        for (int b = 0; b < (int)x->bcs.size(); b++) {
            k_tape_ring<<<gr, 256, 0, s>>>(dc, x->P, x->tape, b);
            k_bc_one<double, NQ><<<gb, 256, 0, s>>>(dc, x->P, b, 0);
            if (x->bcs[b].type == ST_BC_WAKE) k_bc_one<double, NQ><<<gb, 256, 0, s>>>(dc, x->P, b, 1);
        }
        if (dc.viscous) k_bc_mu<double, NQ><<<gr, 256, 0, s>>>(dc, x->P);
    }
    stx::mark(x, "k_bc_taped");
    if (ORDER == 2) {
        k_limiter<double, NQ, true><<<gc, 256, 0, s>>>(dc, x->P, x->lim);
        stx::mark(x, "k_limiter_adj");
    }
    if (NQ == 5 && dc.viscous) {
        k_face_grad<0><<<grid_for(x->nfi), 256, 0, s>>>(dc, x->P, x->Gi);
        k_face_grad<1><<<grid_for(x->nfj), 256, 0, s>>>(dc, x->P, x->Gj);
        stx::mark(x, "k_face_grad(i+j)");
    }
    // psi is first read below: a host-buffer call copies it in meanwhile
    if (x->hio.psi_ready) ST_CUDA(cudaStreamWaitEvent(s, x->hio.psi_ready, 0));
    if (NQ == 5 && dc.viscous) {
        k_cell_src<<<gc, 256, 0, s>>>(dc, x->P, x->Gi, x->Gj, x->beta, psi, x->srec, outb);
        stx::mark(x, "k_cell_src");
    }
    if (x->hio.outb) {  // outb is final (set above or zeroed before the pipeline)
        const int rc = stx::copy_out(x, x->xev[2], x->hio.outb, outb, x->ncell * 8);
        if (rc) return rc;
    }
    k_face_fused<NQ, 0, ORDER, FLUX><<<grid_for(x->nfi), 256, 0, s>>>(dc, x->P, x->lim, psi, x->srec, rhs ? x->Fi : nullptr,
                                                                x->arec_i);
    stx::mark(x, "k_face_fused_i");
    k_face_fused<NQ, 1, ORDER, FLUX><<<grid_for(x->nfj), 256, 0, s>>>(dc, x->P, x->lim, psi, x->srec, rhs ? x->Fj : nullptr,
                                                                x->arec_j);
    stx::mark(x, "k_face_fused_j");
    if (rhs) {
        k_cell_res<NQ><<<gc, 256, 0, s>>>(dc, x->Fi, x->Fj, x->srec, rhs);
        stx::mark(x, "k_cell_res");
        if (x->hio.rhs) {  // copied out while the gather runs
            const int rc = stx::copy_out(x, x->xev[3], x->hio.rhs, rhs, x->ncell * NQ * 8);
            if (rc) return rc;
        }
    }
    const unsigned gr = (unsigned)((2 * (x->c.ni + 1) + 2 * (x->c.nj - 1) + 255) / 256);
    const unsigned gb = (unsigned)((std::max(x->c.ni, x->c.nj) + 1 + 255) / 256);
    auto bc_reverse = [&]() {
        if (dc.viscous) k_bc_adj_mu<NQ><<<gr, 256, 0, s>>>(dc, x->P, x->Pbar);
        for (int b = (int)x->bcs.size() - 1; b >= 0; b--) {
            k_bc_adj_one<NQ><<<gb, 256, 0, s>>>(dc, x->P, x->tape, x->Pbar, b, 0);
            if (x->bcs[b].type == ST_BC_WAKE) k_bc_adj_one<NQ><<<gb, 256, 0, s>>>(dc, x->P, x->tape, x->Pbar, b, 1);
        }
    };
    if (x->hio.outq && x->ring_dev) {
        // host-buffer call: the gather in bands of padded rows, each band's
        // interior state products right behind it and on their way to the
        // host while the next band gathers; the boundary ring, which the
        // boundary reverse still changes, after that reverse, packed
        const int nic = x->c.ni - 1, njc = x->c.nj - 1, nb = st_ctx::kBands;
        const size_t rowp = (size_t)njc + 2;
        for (int b = 0; b < nb; b++) {
            const int r0 = (nic + 2) * b / nb, r1 = (nic + 2) * (b + 1) / nb;
            k_gather<NQ, ORDER><<<grid_for((r1 - r0) * rowp), 256, 0, s>>>(dc, x->P, x->arec_i, x->arec_j, x->srec,
                                                                          x->Pbar, r0 * rowp, r1 * rowp);
            const size_t i0 = (size_t)std::max(r0, 1) - 1, i1 = (size_t)std::min(r1, nic + 1) - 1;
            if (i1 > i0) {
                k_prim_adj<NQ><<<grid_for((i1 - i0) * njc), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, outq, i0 * njc,
                                                                        i1 * njc, true);
                const int rc = stx::copy_out(x, x->band_ev[b], x->hio.outq + i0 * njc * NQ, outq + i0 * njc * NQ,
                                             (i1 - i0) * njc * NQ * 8);
                if (rc) return rc;
            }
        }
        stx::mark(x, "k_gather");
        bc_reverse();
        stx::mark(x, "k_bc_adj");
        const size_t nr = ring_cells(nic, njc);
        k_prim_adj_ring<NQ><<<grid_for(nr), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, outq, x->ring_dev);
        stx::mark(x, "k_prim_adj");
        const int rc = stx::copy_out(x, x->xev[4], x->ring_host, x->ring_dev, nr * NQ * 8);
        if (rc) return rc;
        x->ring_pending = true;
    } else {
        k_gather<NQ, ORDER><<<grid_for(x->npad), 256, 0, s>>>(dc, x->P, x->arec_i, x->arec_j, x->srec, x->Pbar, 0,
                                                            x->npad);
        stx::mark(x, "k_gather");
        bc_reverse();
        stx::mark(x, "k_bc_adj");
        const int rc = stx::run_banded(x, x->hio.outq, outq, NQ, [&](size_t f, size_t l) {
            k_prim_adj<NQ><<<grid_for(l - f), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, outq, f, l);
        });
        if (rc) return rc;
        stx::mark(x, "k_prim_adj");
    }
    ST_LAUNCH_CHECK("residual/adjoint launch");
    return ST_OK;
}

// launches of the grid-wide boundary pass: one per BC (two for a wake cut),
// plus the ghost viscosities when viscous
int bc_launches(const st_ctx* x) {
    int n = 0;
    for (const auto& b : x->bcs) n += b.type == ST_BC_WAKE ? 2 : 1;
    return n + (x->dc.viscous ? 1 : 0);
}

int fused_launches(const st_ctx* x, int order, bool with_rhs) {
    int n = 5;  // prim, face x2, gather, prim_adj
    n += bc_launches(x) + (int)x->bcs.size();  // taped boundary pass: a ring copy before each BC
    n += bc_launches(x);                        // its reverse
    if (order == 2) n += 1;
    if (x->nq == 5 && x->dc.viscous) n += 3;
    if (with_rhs) n += 1;
    return n;
}

template <int FLUX>
int run_fused_flux(st_ctx* x, const double* psi, double* rhs, double* outq, double* outb, int order) {
    if (x->nq == 5)
        return order == 2 ? launch_fused<5, 2, FLUX>(x, psi, rhs, outq, outb) : launch_fused<5, 1, FLUX>(x, psi, rhs, outq, outb);
    return order == 2 ? launch_fused<4, 2, FLUX>(x, psi, rhs, outq, outb) : launch_fused<4, 1, FLUX>(x, psi, rhs, outq, outb);
}

int run_fused(st_ctx* x, const double* psi, double* rhs, double* outq, double* outb, int lhs) {
    int rc = ensure(x);
    if (rc) return rc;
    const int order = lhs ? x->c.lhs_order : x->c.order;
    if (x->nq == 4 || !x->dc.viscous) ST_CUDA(cudaMemsetAsync(outb, 0, x->ncell * 8, x->stream));
    return x->c.flux == ST_FLUX_AUSM ? run_fused_flux<ST_FLUX_AUSM>(x, psi, rhs, outq, outb, order)
                                     : run_fused_flux<ST_FLUX_ROE>(x, psi, rhs, outq, outb, order);
}

}  // namespace

namespace stx {
int ensure_adjoint_buffers(st_ctx* x) { return ensure(x); }
}  // namespace stx

namespace {
// Enqueues a host-buffer VJP with its copies overlapped (see host_vjp).
int host_vjp_enqueue(st_ctx* x, const double* psi_host, double* rhs_host, double* outq_host, double* outb_host,
                     int lhs, bool with_rhs) {
    const size_t nqb = x->ncell * x->nq * 8;
    // the copy stream starts after the work already queued (which may still read psi_tmp)
    ST_CUDA(cudaEventRecord(x->xev[0], x->stream));
    ST_CUDA(cudaStreamWaitEvent(x->xfer, x->xev[0], 0));
    ST_CUDA(cudaMemcpyAsync(x->psi_tmp, psi_host, nqb, cudaMemcpyHostToDevice, x->xfer));
    ST_CUDA(cudaEventRecord(x->xev[1], x->xfer));
    x->hio.psi_ready = x->xev[1];
    x->hio.rhs = with_rhs ? rhs_host : nullptr;
    x->hio.outq = outq_host;
    x->hio.outb = outb_host;
    const int rc = with_rhs ? st_residual_vjp_device(x, x->psi_tmp, x->rhs, x->outq_tmp, x->outb_tmp, lhs)
                            : st_vjp_device(x, x->psi_tmp, x->outq_tmp, x->outb_tmp, lhs);
    x->hio = {};
    if (rc) return rc;
    if (with_rhs) x->have_residual = true;
    return ST_OK;
}

// Host-buffer VJP (and residual): psi goes in on the copy stream while the
// forward passes run, and the pipeline waits for it before its first read of
// psi; the beta product and the residual go out on that stream as soon as
// they are final, during the gather.  The gather runs in bands, each followed
// by k_prim_adj on the band's interior cells, whose state products go out
// while the next band gathers; the boundary ring follows the boundary reverse
// and is copied packed, then scattered into out_q_host here (small grids: the
// gather whole, then k_prim_adj in bands).  Both streams are drained before
// the call returns, on errors too, so the caller's buffers are free again.
int host_vjp(st_ctx* x, const double* psi_host, double* rhs_host, double* outq_host, double* outb_host, int lhs,
             bool with_rhs) {
    int rc = ensure(x);
    if (rc) return rc;
    x->ring_pending = false;
    rc = host_vjp_enqueue(x, psi_host, rhs_host, outq_host, outb_host, lhs, with_rhs);
    const cudaError_t e1 = cudaStreamSynchronize(x->xfer);
    const cudaError_t e2 = cudaStreamSynchronize(x->stream);
    const bool ring = x->ring_pending;
    x->ring_pending = false;
    if (rc) return rc;
    if (e1 != cudaSuccess) return stx::cuda_fail(e1, "cudaStreamSynchronize (copy stream)");
    if (e2 != cudaSuccess) return stx::cuda_fail(e2, "cudaStreamSynchronize");
    if (ring) {  // the boundary ring of the state product into its place in out_q_host
        const int nic = x->c.ni - 1, njc = x->c.nj - 1, nq = x->nq;
        const size_t nr = ring_cells(nic, njc);
        for (size_t r = 0; r < nr; r++)
            std::memcpy(outq_host + ring_cell(nic, njc, r) * nq, x->ring_host + r * nq, nq * sizeof(double));
    }
    return ST_OK;
}
}  // namespace

extern "C" {

int st_vjp_device(st_ctx* x, const double* psi, double* outq, double* outb, int lhs) {
    if (!x || !psi) return fail(ST_ERR_ARG, "st_vjp_device: null argument");
    int rc = ensure(x);
    if (rc) return rc;
    cudaEventRecord(x->ev[2], x->stream);
    rc = run_fused(x, psi, nullptr, outq ? outq : x->outq_tmp, outb ? outb : x->outb_tmp, lhs);
    if (rc) return rc;
    cudaEventRecord(x->ev[3], x->stream);
    x->vjp_pending = true;
    return ST_OK;
}

int st_residual_vjp_device(st_ctx* x, const double* psi, double* rhs, double* outq, double* outb, int lhs) {
    if (!x || !psi || !rhs) return fail(ST_ERR_ARG, "st_residual_vjp_device: null argument");
    int rc = ensure(x);
    if (rc) return rc;
    cudaEventRecord(x->ev[2], x->stream);
    rc = run_fused(x, psi, rhs, outq ? outq : x->outq_tmp, outb ? outb : x->outb_tmp, lhs);
    if (rc) return rc;
    cudaEventRecord(x->ev[3], x->stream);
    x->vjp_pending = true;
    return ST_OK;
}

int st_vjp(st_ctx* x, const double* psi_host, double* outq_host, double* outb_host, int lhs) {
    if (!x || !psi_host) return fail(ST_ERR_ARG, "st_vjp: null argument");
    return host_vjp(x, psi_host, nullptr, outq_host, outb_host, lhs, false);
}

int st_residual_vjp(st_ctx* x, const double* psi_host, double* rhs_host, double* outq_host, double* outb_host, int lhs) {
    if (!x || !psi_host) return fail(ST_ERR_ARG, "st_residual_vjp: null argument");
    return host_vjp(x, psi_host, rhs_host, outq_host, outb_host, lhs, true);
}

int st_launch_counts(st_ctx* x, int lhs, int* residual, int* vjp) {
    if (!x) return fail(ST_ERR_ARG, "st_launch_counts: null context");
    const int order = lhs ? x->c.lhs_order : x->c.order;
    if (residual) {
        // prim, the boundary pass, then the two tiled sweeps or the per-stage passes
        const bool tiled = x->tile_ok && x->res_path == 1 && !x->dc.mlp_wb;
        *residual = 1 + bc_launches(x) + (tiled ? 2 : (order == 2 ? 4 : 3));
    }
    if (vjp) *vjp = fused_launches(x, order, false);
    return ST_OK;
}

int st_fused_launch_count(st_ctx* x, int lhs) {
    if (!x) return fail(ST_ERR_ARG, "st_fused_launch_count: null context");
    return fused_launches(x, lhs ? x->c.lhs_order : x->c.order, true);
}

}  // extern "C"
