// Host build of structured_gb300/csrc/st_wake.cuh (test infrastructure): the
// same kernel source compiled by g++, each launch run serially as one block of
// one thread, so that the CPU tests can check the wake column mask, the
// partner seeds and extraction, and the partner products against the oracle
// and catch any index outside its buffer.
#define __global__
#define __device__
#define __host__
struct HostDim3 {
    int x;
};
static const HostDim3 blockIdx{0}, threadIdx{0}, blockDim{1}, gridDim{1};

#include "../structured_gb300/csrc/st_wake.cuh"

using namespace st;

extern "C" {

int wh_slots() { return NWS; }

int wh_columns(int nic, int njc, const st_bc* bcs, int nbc, int* mask, int* any) {
    const char* why = "";
    return wake_columns(nic, njc, bcs, nbc, mask, any, &why);
}

void wh_seed(int nq, int nic, int njc, const int* mask, int side, int k, int comp, double* v) {
    if (nq == 5) k_wake_seed<5>(nic, njc, mask, side, k, comp, v);
    else k_wake_seed<4>(nic, njc, mask, side, k, comp, v);
}

void wh_extract(int nq, int nic, int njc, const int* mask, int side, int k, int comp, const double* jv,
                double* W) {
    if (nq == 5) k_wake_extract<5>(nic, njc, mask, side, k, comp, jv, W);
    else k_wake_extract<4>(nic, njc, mask, side, k, comp, jv, W);
}

void wh_apply(int nq, int trans, int nic, int njc, const double* W, const double* x, double* y, double sj) {
    if (nq == 5) {
        if (trans) k_wake_apply<5, true>(nic, njc, W, x, y, sj);
        else k_wake_apply<5, false>(nic, njc, W, x, y, sj);
    } else {
        if (trans) k_wake_apply<4, true>(nic, njc, W, x, y, sj);
        else k_wake_apply<4, false>(nic, njc, W, x, y, sj);
    }
}

}  // extern "C"
