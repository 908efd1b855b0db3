// Host-side helpers shared by the reduced-basis plans (vd_basis.cu,
// vd_basis_bm.cu): the reference's lattice formulas use Python / NumPy
// arithmetic, reproduced here value for value.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace vd {
namespace basis_host {

// Python float modulo (result has the sign of the divisor).
inline double pymod(double a, double b)
{
    double r = std::fmod(a, b);
    if (r != 0.0 && ((r < 0.0) != (b < 0.0))) r += b;
    return r;
}

// numpy.arange(start, stop, step) for float64: length ceil((stop-start)/step),
// values start, start+step, then start + i*((start+step)-start).
inline std::vector<double> np_arange(double start, double stop, double step)
{
    const double len = std::ceil((stop - start) / step);
    const long n = len > 0 ? (long)len : 0;
    std::vector<double> v((size_t)n);
    if (n > 0) v[0] = start;
    if (n > 1) v[1] = start + step;
    const double delta = (start + step) - start;
    for (long i = 2; i < n; ++i) v[(size_t)i] = start + (double)i * delta;
    return v;
}

// numpy.linspace(start, stop, num) for float64.
inline std::vector<double> np_linspace(double start, double stop, int num)
{
    std::vector<double> v((size_t)num);
    if (num == 1) {
        v[0] = start;
        return v;
    }
    const double step = (stop - start) / (num - 1);
    for (int i = 0; i < num; ++i) v[(size_t)i] = (double)i * step + start;
    v[(size_t)num - 1] = stop;
    return v;
}

// cos^2 window and flux window (mapping/src/basis.py:4138-4144)
inline double mywindow(double x)
{
    const double c = std::cos(x * 0.5 * M_PI);
    return c * c;
}
inline double mywindow_flux(double x)
{
    return -M_PI * std::sin(x * 0.5 * M_PI) * std::cos(x * 0.5 * M_PI);
}

// max of the cumulative trapezoid of the window over linspace(-T, T, 50)
// (basis.py:1278-1283, 662-666)
template <typename W>
inline double window_norm(double T, W window)
{
    const std::vector<double> tt = np_linspace(-T, T, 50);
    double tmp = 0.0, mx = 0.0;
    for (size_t i = 0; i + 1 < tt.size(); ++i) {
        tmp = tmp + window(tt[i] / T) * (tt[i + 1] - tt[i]);
        mx = std::max(mx, tmp);
    }
    return mx;
}

// Packs host vectors into one device allocation; returns device pointers.
struct Packer {
    std::vector<unsigned char> blob;
    template <typename V>
    size_t add(const std::vector<V>& v)
    {
        size_t off = (blob.size() + 255) & ~size_t(255);
        blob.resize(off + v.size() * sizeof(V) + 1);
        if (!v.empty()) std::memcpy(blob.data() + off, v.data(), v.size() * sizeof(V));
        return off;
    }
    template <typename T>
    size_t add_as(const std::vector<double>& v)
    {
        std::vector<T> t(v.begin(), v.end());
        return add(t);
    }
};


}  // namespace basis_host
}  // namespace vd
