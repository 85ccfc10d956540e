// Hand-written discrete adjoint (reverse mode) of the residual pipeline.
#include "st_context.h"
#include "st_kernels.cuh"

extern "C" {
int st_vjp_device(st_ctx* x, const double*, double*, double*, int) {
    if (!x) return stx::fail(ST_ERR_ARG, "st_vjp_device: null context");
    return stx::fail(ST_ERR_UNSUPPORTED, "st_vjp_device: not built yet");
}
int st_vjp(st_ctx* x, const double*, double*, double*, int) {
    if (!x) return stx::fail(ST_ERR_ARG, "st_vjp: null context");
    return stx::fail(ST_ERR_UNSUPPORTED, "st_vjp: not built yet");
}
}
