// Host build of the tracer point rules of the GPU kernels
// (vardyn_gb300/csrc/vd_qgtrac.cuh), looped over whole planes so that a CPU
// test can compare them with the oracle. Test infrastructure only.
#include "../vardyn_gb300/csrc/vd_qgtrac.cuh"

extern "C" void trac_rhs_plane_f64(int ny, int nx, double dx, double dy, int hasK, double K, const int8_t* mask,
                                   const double* u, const double* v, const double* c, double* out)
{
    vd::TracGeom G{};
    G.ny = ny; G.nx = nx;
    G.cx = 1.0 / (6.0 * dx); G.cy = 1.0 / (6.0 * dy);
    G.hasK = hasK; G.Kx = hasK ? K / (dx * dx) : 0.0; G.Ky = hasK ? K / (dy * dy) : 0.0;
    G.mask = mask;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) out[(long long)j * nx + i] = vd::trac_rhs_point<double>(G, u, v, c, j, i);
}

extern "C" void trac_bc_plane_f64(int ny, int nx, double dx, double dy, double dt, int obc, const int8_t* mask,
                                  const double* u, const double* v, const double* a, const double* b,
                                  const double* W, double* x)
{
    vd::TracGeom G{};
    G.ny = ny; G.nx = nx;
    G.rx = 0.5 * dt / dx; G.ry = 0.5 * dt / dy;
    G.obc = obc;
    G.mask = mask;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const long long o = (long long)j * nx + i;
            x[o] = vd::trac_bc_point<double>(G, u, v, a, b, W, x[o], j, i);
        }
}

extern "C" double rk_combine_f64(int mode, double a, double dt, double r, double base, double* acc)
{
    return vd::rk_combine<double>(mode, a, dt, r, base, acc);
}
