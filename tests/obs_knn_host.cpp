// Host build of the observation neighbour search of the GPU kernel
// (vardyn_gb300/csrc/vd_obs_knn.cuh), looped over observations, so that a
// CPU test can compare it with the oracle. Test infrastructure only.
#include "../vardyn_gb300/csrc/vd_obs_knn.cuh"

extern "C" void obs_knn_host(long long nobs, const double* x, const double* y, int ny, int nx, double dx, double dy,
                             int npix, double dmax, const unsigned char* excl, long long* idx, double* w)
{
    for (long long o = 0; o < nobs; ++o)
        vd::obs_knn_point(x[o], y[o], ny, nx, dx, dy, npix, dmax, excl, idx + o * 4, w + o * 4);
}
