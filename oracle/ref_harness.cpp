/* Test infrastructure: a C entry layer over the reference solver's own
 * residual code (anandpratap/structured, src/), compiled out of tree.
 *
 * Only tests, the smoke check and bench.py's CPU-baseline leg load the library
 * built from this file.  It drives, unmodified:
 *   Config<double>             src/utils/config.cpp:104-123 (TOML case setup)
 *   Mesh<double,double>        src/utils/mesh.cpp:345-414 (grid load, metrics, setup)
 *   EulerEquation::calc_residual  src/model/eulerequation.cpp:202-232
 *   EulerEquation::calc_dt        src/model/eulerequation.cpp:237-259
 * and copies state in and residuals out through flat arrays in the
 * reference's q[i][j][k] layout (src/solver/solution.cpp:28). */
#include "common.h"
#include "config.h"
#include "mesh.h"
#include "solution.h"
#include "eulerequation.h"
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {
struct RefCase {
    std::shared_ptr<Config<double>> config;
    std::shared_ptr<Mesh<double, double>> mesh;
};
std::shared_ptr<spdlog::logger> ensure_logger() {
    auto lg = spdlog::get("console");
    if (!lg) lg = spdlog::stdout_logger_mt("console", true);
    lg->set_level(spdlog::level::err);
    return lg;
}
}  // namespace

extern "C" {

void* refh_open(const char* inp_path) {
    try {
        spdlog::set_pattern("%v");
        ensure_logger();
        char* argv0[] = {(char*)"ref", nullptr};
        auto* rc = new RefCase();
        rc->config = std::make_shared<Config<double>>(std::string(inp_path), 1, argv0);
        rc->mesh = std::make_shared<Mesh<double, double>>(rc->config);
        rc->mesh->label = "";
        rc->mesh->setup();
        return rc;
    } catch (...) {
        return nullptr;
    }
}

void refh_close(void* h) { delete static_cast<RefCase*>(h); }

int refh_dims(void* h, int* ni, int* nj, int* nq) {
    auto* rc = static_cast<RefCase*>(h);
    *ni = (int)rc->mesh->ni;
    *nj = (int)rc->mesh->nj;
    *nq = (int)(rc->mesh->solution->nq + rc->mesh->solution->ntrans);
    return 0;
}

int refh_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* q and rhs: [nic][njc][nq] row-major doubles.  lhs selects the reference's
 * lhs_order reconstruction (src/model/eulerequation.cpp:203-208). */
int refh_residual(void* h, const double* q, double* rhs, int lhs) {
    auto* rc = static_cast<RefCase*>(h);
    auto sol = rc->mesh->solution;
    const size_t n = sol->q.size();
    std::memcpy(sol->q.data(), q, n * sizeof(double));
    rc->mesh->equation->calc_residual(sol->q.const_ref(), sol->rhs, lhs != 0);
    std::memcpy(rhs, sol->rhs.data(), n * sizeof(double));
    return 0;
}

/* Residual on the state already loaded (timing loop without copies). */
int refh_residual_inplace(void* h, int lhs) {
    auto* rc = static_cast<RefCase*>(h);
    auto sol = rc->mesh->solution;
    rc->mesh->equation->calc_residual(sol->q.const_ref(), sol->rhs, lhs != 0);
    return 0;
}

int refh_dt(void* h, const double* q, double cfl, double* dt) {
    auto* rc = static_cast<RefCase*>(h);
    auto sol = rc->mesh->solution;
    const size_t n = sol->q.size();
    std::memcpy(sol->q.data(), q, n * sizeof(double));
    rc->mesh->equation->calc_dt(cfl);
    std::memcpy(dt, sol->dt.data(), n * sizeof(double));
    return 0;
}

/* Mesh metrics (src/utils/mesh.cpp:172-205): normal_chi [ni][njc][2],
 * normal_eta [nic][nj][2], volume [nic][njc]. */
int refh_metrics(void* h, double* normal_chi, double* normal_eta, double* volume) {
    auto* rc = static_cast<RefCase*>(h);
    auto m = rc->mesh;
    std::memcpy(normal_chi, m->normal_chi.data(), m->normal_chi.size() * sizeof(double));
    std::memcpy(normal_eta, m->normal_eta.data(), m->normal_eta.size() * sizeof(double));
    std::memcpy(volume, m->volume.data(), m->volume.size() * sizeof(double));
    return 0;
}

/* Ghost-padded primitives after primvars + boundary conditions of the last
 * residual call (src/model/eulerequation.cpp:157-173): five arrays
 * [nic+2][njc+2] packed back to back as rho, u, v, p, T. */
int refh_primitives(void* h, double* out) {
    auto* rc = static_cast<RefCase*>(h);
    auto eq = rc->mesh->equation;
    const size_t n = eq->rho.size();
    std::memcpy(out + 0 * n, eq->rho.data(), n * sizeof(double));
    std::memcpy(out + 1 * n, eq->u.data(), n * sizeof(double));
    std::memcpy(out + 2 * n, eq->v.data(), n * sizeof(double));
    std::memcpy(out + 3 * n, eq->p.data(), n * sizeof(double));
    std::memcpy(out + 4 * n, eq->T.data(), n * sizeof(double));
    return 0;
}

/* j-face gradients of u and v of the last residual call (u_x,u_y,v_x,v_y per
 * face, [nic][nj][4]); the reference's wall skin friction reads the j=0 row
 * of these (src/utils/io.cpp:217-224). */
int refh_eta_gradients(void* h, double* out) {
    auto* rc = static_cast<RefCase*>(h);
    auto eq = rc->mesh->equation;
    const size_t nic = rc->mesh->nic, nj = rc->mesh->nj;
    for (size_t i = 0; i < nic; i++)
        for (size_t j = 0; j < nj; j++) {
            double* o = out + (i * nj + j) * 4;
            o[0] = eq->grad_u_eta[i][j][0];
            o[1] = eq->grad_u_eta[i][j][1];
            o[2] = eq->grad_v_eta[i][j][0];
            o[3] = eq->grad_v_eta[i][j][1];
        }
    return 0;
}

/* IOManager::write (src/utils/io.cpp:41-47) on state q: the reference writes
 * <io.label>.tec, .npz, .out and .surface.  The residual of q is evaluated
 * first (as Solver::step has done before it writes) so the wall-face
 * gradients the surface file reads belong to q. */
int refh_write_outputs(void* h, const double* q) {
    auto* rc = static_cast<RefCase*>(h);
    auto sol = rc->mesh->solution;
    std::memcpy(sol->q.data(), q, sol->q.size() * sizeof(double));
    rc->mesh->equation->calc_residual(sol->q.const_ref(), sol->rhs);
    rc->mesh->iomanager->write(0);
    return 0;
}

}  // extern "C"
