// Host build of structured_gb300/csrc/st_partner.cuh (test infrastructure):
// the same kernel source compiled by g++, each launch run serially as one
// block of one thread, so that the CPU tests can check the ghost masks, the
// partner seeds and extraction, and the partner products against the oracle
// and catch any index outside its buffer.
#define __global__
#define __device__
#define __host__
struct HostDim3 {
    int x;
};
static const HostDim3 blockIdx{0}, threadIdx{0}, blockDim{1}, gridDim{1};

#include "../structured_gb300/csrc/st_partner.cuh"

using namespace st;

extern "C" {

int ph_slots() { return NWS; }

int ph_masks(int nic, int njc, const st_bc* bcs, int nbc, int* mask_wake, int* mask_left, int* mask_right,
             int* on) {
    const char* why = "";
    return partner_masks(nic, njc, bcs, nbc, mask_wake, mask_left, mask_right, on, &why);
}

void ph_seed(int nq, int f, int nic, int njc, const int* mask, int k, int comp, double* v) {
    if (nq == 5) k_partner_seed<5>(f, nic, njc, mask, k, comp, v);
    else k_partner_seed<4>(f, nic, njc, mask, k, comp, v);
}

void ph_extract(int nq, int f, int nic, int njc, const int* mask, int k, int comp, const double* jv_full,
                const double* jv_frozen, double* W) {
    if (nq == 5) k_partner_extract<5>(f, nic, njc, mask, k, comp, jv_full, jv_frozen, W);
    else k_partner_extract<4>(f, nic, njc, mask, k, comp, jv_full, jv_frozen, W);
}

void ph_apply(int nq, int trans, int f, int nic, int njc, const double* W, const double* x, double* y, double sj) {
    if (nq == 5) {
        if (trans) k_partner_apply<5, true>(f, nic, njc, W, x, y, sj);
        else k_partner_apply<5, false>(f, nic, njc, W, x, y, sj);
    } else {
        if (trans) k_partner_apply<4, true>(f, nic, njc, W, x, y, sj);
        else k_partner_apply<4, false>(f, nic, njc, W, x, y, sj);
    }
}

int ph_off13(int di, int dj) { return off13(di, dj); }

void ph_fold(int nq, int f, int nic, int njc, const double* W, double* jac) {
    if (nq == 5) k_partner_fold<5>(f, nic, njc, W, jac);
    else k_partner_fold<4>(f, nic, njc, W, jac);
}

int ph_strip_cells(int nic, int njc, const int* mask_wake, int* cells) {
    return strip_cells(nic, njc, mask_wake, cells);
}

void ph_strip_matrix(int nic, int njc, int nq, int ns, const int* cells, const double* jac_s, const double* dt_s,
                     const double* W1, double psd, double sj, double* A) {
    strip_matrix(nic, njc, nq, ns, cells, jac_s, dt_s, W1, psd, sj, A);
}

int ph_dense_invert(int n, double* A, double* inv) { return dense_invert(n, A, inv); }

void ph_strip_gather(int nq, int ns, const int* cells, const double* jac, const double* dt, double* jac_s,
                     double* dt_s) {
    if (nq == 5) k_strip_gather<5>(ns, cells, jac, dt, jac_s, dt_s);
    else k_strip_gather<4>(ns, cells, jac, dt, jac_s, dt_s);
}

void ph_strip_residual(int nq, int nic, int njc, int ns, const int* cells, const double* jac, const double* W1,
                       const double* dt, double psd, double sj, const double* v, const double* z, double* res) {
    if (nq == 5) k_strip_residual<5>(nic, njc, ns, cells, jac, W1, dt, psd, sj, v, z, res);
    else k_strip_residual<4>(nic, njc, ns, cells, jac, W1, dt, psd, sj, v, z, res);
}

void ph_strip_update(int nq, int ns, const int* cells, const double* Ainv, const double* res, double* z) {
    if (nq == 5) k_strip_update<5>(ns, cells, Ainv, res, z);
    else k_strip_update<4>(ns, cells, Ainv, res, z);
}

}  // extern "C"
