// Wave-packet reduced basis (Basis_bm / Basis_bm_jax, mapping/src/basis.py
// 472-1168): phi = G(t) X and adX += G(t)^T adphi.
//
// Frequencies ff (577-583), directions theta (587), per frequency a lattice of
// centres (611-649) and atoms
//   sqrt(2) w(xx/DX) w(yy/DX) {cos, sin}(kx xx + ky yy),  w = cos^2 window,
// kx = k cos(theta), ky = k sin(theta), k = 2 pi ff (736-772). With
// cos(A + B) = cos A cos B - sin A sin B and sin(A + B) = sin A cos B +
// cos A sin B every atom is a sum of two separable products, so G is two
// banded passes with two channels per direction (no sparse matrix, no
// atomics):
//   x pass  T1[r][th][x] = sum_i wx (cos A Zc + sin A Zs)
//           T2[r][th][x] = sum_i wx (cos A Zs - sin A Zc)
//   y pass  phi[y][x]    = sum_f sum_th sum_j sqrt(2) wy (cos B T1 + sin B T2)
// where Z{c,s}(i, th) = sum over active time centres of g_it X[it][i][th][c|s].
// The transpose runs the passes backwards. Coefficients of one frequency are
// ordered [time centre][space centre][theta][cos, sin] (basis.py:775-781).
#include "vd_internal.cuh"
#include "vd_basis_host.h"
#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <vector>

namespace {

using namespace vd::basis_host;

struct BmFreq {
    double ff = 0, k = 0, DX = 0, DXG = 0, tdec = 0, norm_fact = 1, Q = 0;
    std::vector<double> enst;
    std::vector<double> tscale, tnorm;   // wavelet basis: per time centre DXt and norm_fact
    std::vector<double> rows_lat;
    std::vector<std::vector<double>> row_lons;
    std::vector<double> enslat, enslon;
    long long NP = 0;
    long long boff = 0;
    int rowoff = 0;
    // auxiliary-field basis: per space centre the decorrelation time, window
    // integral, time-centre axis (numpy arange: start, start + step, then
    // start + i * delta) and count, prior std; the padded time-centre count
    std::vector<double> c_tdec, c_norm, c_start, c_step, c_delta, c_std;
    std::vector<int> c_n;
    int nit = 0;
    long long cboff = 0, cstart = 0;
};

}  // namespace

struct vd_bm_plan {
    int ny = 0, nx = 0, dtype = VD_F32, geographic = 0, host_only = 0, ntime = 0;
    int nf = 0, nth = 0;
    long long nbasis = 0;
    int R = 0, KX = 1, KY = 1, NA = 1;
    vd_bm_params prm;
    int kind = 0;                 // 0 wave packets (Basis_bm), 1 wavelets (Basis_wavelet3d),
                                  // 2 wave packets with auxiliary fields (Basis_bmaux)
    vd_wavelet_params wprm;
    vd_bmaux_params aprm;
    std::vector<double> ax_f, ax_lat, ax_lon, ax_td, ax_sd;
    long long cbasis = 0;         // kind 2: time-reduced coefficients per window
    long long ncentres = 0;
    void* dev_aux = nullptr;
    const double* d_ctab = nullptr;   // kind 2: [centre][5] tdec, norm, start, step, delta
    const int32_t* d_cn = nullptr;    // kind 2: [centre] time-centre count
    std::vector<double> theta;
    std::vector<BmFreq> fr;
    std::vector<double> times;
    std::vector<int> tact_n, tact_it;
    std::vector<double> tact_g;
    void* dev = nullptr;
    const int32_t *row_freq, *row_pat, *row_n, *fx_i, *tx_ptr, *tx_x, *tx_e, *pat_cbase, *fy_j, *ty_ptr, *ty_y,
        *ty_e, *freq_rowoff, *d_tact_n, *d_tact_it;
    const long long *row_cb, *freq_boff, *freq_np;
    const void *fx_c, *fx_s, *fy_c, *fy_s, *d_tact_g;
    const int8_t* land;
};

namespace vd {

template <typename T>
struct BmDev {
    int ny, nx, R, KX, KY, NA, nf, nth;
    const int32_t *row_freq, *row_pat, *row_n, *fx_i, *tx_ptr, *tx_x, *tx_e, *pat_cbase, *fy_j, *ty_ptr, *ty_y,
        *ty_e, *freq_rowoff, *tact_n, *tact_it;
    const long long *row_cb, *freq_boff, *freq_np;
    const T *fx_c, *fx_s, *fy_c, *fy_s, *tact_g;
    const int8_t* land;
};

template <typename T>
BmDev<T> bm_view(const vd_bm_plan* p)
{
    BmDev<T> d;
    d.ny = p->ny; d.nx = p->nx; d.R = p->R; d.KX = p->KX; d.KY = p->KY; d.NA = p->NA; d.nf = p->nf;
    d.nth = p->nth;
    d.row_freq = p->row_freq; d.row_pat = p->row_pat; d.row_n = p->row_n; d.fx_i = p->fx_i;
    d.tx_ptr = p->tx_ptr; d.tx_x = p->tx_x; d.tx_e = p->tx_e; d.pat_cbase = p->pat_cbase;
    d.fy_j = p->fy_j; d.ty_ptr = p->ty_ptr; d.ty_y = p->ty_y; d.ty_e = p->ty_e; d.freq_rowoff = p->freq_rowoff;
    d.tact_n = p->d_tact_n; d.tact_it = p->d_tact_it;
    d.row_cb = p->row_cb; d.freq_boff = p->freq_boff; d.freq_np = p->freq_np;
    d.fx_c = (const T*)p->fx_c; d.fx_s = (const T*)p->fx_s; d.fy_c = (const T*)p->fy_c;
    d.fy_s = (const T*)p->fy_s; d.tact_g = (const T*)p->d_tact_g;
    d.land = p->land;
    return d;
}

// x pass of G: one thread per (column x, lattice row r and direction th, window b)
template <typename T>
__global__ void __launch_bounds__(128)
k_bm_xpass(BmDev<T> d, int k, const T* __restrict__ X, long long ldX, T* __restrict__ Tw)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int rt = blockIdx.y, b = blockIdx.z;
    if (x >= d.nx) return;
    const int r = rt / d.nth, th = rt - r * d.nth;
    const int f = d.row_freq[r], p = d.row_pat[r];
    const long long stride = 2LL * d.nth * d.freq_np[f];
    const T* Xr = X + (long long)b * ldX + d.freq_boff[f] + (d.row_cb[r] * d.nth + th) * 2;
    const int ta = (k * d.nf + f) * d.NA, na = d.tact_n[k * d.nf + f];
    const long long e0 = ((long long)p * d.nx + x) * d.KX;
    const long long w0 = (((long long)p * d.nth + th) * d.nx + x) * d.KX;
    T t1 = T(0), t2 = T(0);
    for (int e = 0; e < d.KX; ++e) {
        const int i = d.fx_i[e0 + e];
        if (i < 0) break;
        T zc = T(0), zs = T(0);
        for (int a = 0; a < na; ++a) {
            const T g = d.tact_g[ta + a];
            const long long o = d.tact_it[ta + a] * stride + (long long)i * 2 * d.nth;
            zc += g * Xr[o];
            zs += g * Xr[o + 1];
        }
        const T cw = d.fx_c[w0 + e], sw = d.fx_s[w0 + e];
        t1 += cw * zc + sw * zs;
        t2 += cw * zs - sw * zc;
    }
    T* o = Tw + (((long long)b * d.R + r) * d.nth + th) * 2 * d.nx + x;
    o[0] = t1;
    o[d.nx] = t2;
}

// y pass of G: one thread per (x, y, b), summing every frequency and direction
template <typename T>
__global__ void __launch_bounds__(128)
k_bm_ypass(BmDev<T> d, const T* __restrict__ Tw, T* __restrict__ phi, int accumulate)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, b = blockIdx.z;
    if (x >= d.nx) return;
    const long long rowstride = (long long)d.nth * 2 * d.nx;
    T acc = T(0);
    for (int f = 0; f < d.nf; ++f) {
        const long long e0 = ((long long)f * d.ny + y) * d.KY;
        for (int th = 0; th < d.nth; ++th) {
            const long long w0 = (((long long)f * d.nth + th) * d.ny + y) * d.KY;
            const T* base = Tw + (((long long)b * d.R + d.freq_rowoff[f]) * d.nth + th) * 2 * d.nx + x;
            for (int e = 0; e < d.KY; ++e) {
                const int j = d.fy_j[e0 + e];
                if (j < 0) break;
                const T* t = base + j * rowstride;
                acc += d.fy_c[w0 + e] * t[0] + d.fy_s[w0 + e] * t[d.nx];
            }
        }
    }
    const long long o = ((long long)b * d.ny + y) * d.nx + x;
    if (d.land && d.land[(long long)y * d.nx + x]) acc = T(0);
    phi[o] = accumulate ? phi[o] + acc : acc;
}

// y pass of G^T: one thread per (x, row r and direction th, b)
template <typename T>
__global__ void __launch_bounds__(128)
k_bmT_ypass(BmDev<T> d, const T* __restrict__ adphi, T* __restrict__ Uw)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int rt = blockIdx.y, b = blockIdx.z;
    if (x >= d.nx) return;
    const int r = rt / d.nth, th = rt - r * d.nth;
    const int f = d.row_freq[r];
    const T* a = adphi + (long long)b * d.ny * d.nx + x;
    T u1 = T(0), u2 = T(0);
    for (int e = d.ty_ptr[r]; e < d.ty_ptr[r + 1]; ++e) {
        const int y = d.ty_y[e];
        const long long w = (((long long)f * d.nth + th) * d.ny + y) * d.KY + d.ty_e[e];
        T v = a[(long long)y * d.nx];
        if (d.land && d.land[(long long)y * d.nx + x]) v = T(0);
        u1 += d.fy_c[w] * v;
        u2 += d.fy_s[w] * v;
    }
    T* o = Uw + (((long long)b * d.R + r) * d.nth + th) * 2 * d.nx + x;
    o[0] = u1;
    o[d.nx] = u2;
}

// x pass of G^T: one CTA per (lattice row r, window b), threads over (centre, direction)
template <typename T>
__global__ void __launch_bounds__(128)
k_bmT_xpass(BmDev<T> d, int k, const T* __restrict__ Uw, T* __restrict__ adX, long long ldX)
{
    const int r = blockIdx.x, b = blockIdx.y;
    const int f = d.row_freq[r], p = d.row_pat[r];
    const long long stride = 2LL * d.nth * d.freq_np[f];
    const int ta = (k * d.nf + f) * d.NA, na = d.tact_n[k * d.nf + f];
    const int base = d.pat_cbase[p];
    T* A = adX + (long long)b * ldX + d.freq_boff[f] + d.row_cb[r] * 2 * d.nth;
    for (int q = threadIdx.x; q < d.row_n[r] * d.nth; q += blockDim.x) {
        const int i = q / d.nth, th = q - i * d.nth;
        const T* U = Uw + (((long long)b * d.R + r) * d.nth + th) * 2 * d.nx;
        T zc = T(0), zs = T(0);
        for (int e = d.tx_ptr[base + i]; e < d.tx_ptr[base + i + 1]; ++e) {
            const int x = d.tx_x[e];
            const long long w = (((long long)p * d.nth + th) * d.nx + x) * d.KX + d.tx_e[e];
            const T u1 = U[x], u2 = U[d.nx + x];
            const T cw = d.fx_c[w], sw = d.fx_s[w];
            zc += cw * u1 - sw * u2;
            zs += sw * u1 + cw * u2;
        }
        for (int a = 0; a < na; ++a) {
            const T g = d.tact_g[ta + a];
            const long long o = d.tact_it[ta + a] * stride + ((long long)i * d.nth + th) * 2;
            A[o] += g * zc;
            A[o + 1] += g * zs;
        }
    }
}

// Auxiliary-field basis, time part at basis time t (days). For space centre
// P of frequency f (global centre index cs + P) the active time centres are
// those with |t - enst| <= tdec_P, weight window((t - enst) / tdec_P) /
// norm_P (basis.py:2337-2352, jax form 2448-2461).
__device__ __forceinline__ double bmaux_weight(const double* tab, int it, double t, int flux)
{
    const double tdec = tab[0], norm = tab[1], start = tab[2], step = tab[3], delta = tab[4];
    const double c = it == 0 ? start : (it == 1 ? start + step : start + (double)it * delta);
    const double dt = t - c;
    if (fabs(dt) > tdec) return 0.0;
    const double x = dt / tdec;
    const double w = flux ? -M_PI * sin(x * 0.5 * M_PI) * cos(x * 0.5 * M_PI)
                          : cos(x * 0.5 * M_PI) * cos(x * 0.5 * M_PI);
    return w / norm;
}

// C[b][cboff + (P nth + th) 2 + c] = sum_it g(it, P) X[b][xboff + ((it NP + P) nth + th) 2 + c]
// for one frequency: one thread per (P, th, c), window b on blockIdx.y
template <typename T>
__global__ void k_bmaux_reduce(const double* __restrict__ ctab, const int32_t* __restrict__ cn, long long cstart,
                               long long np, int nth, long long xboff, long long cboff, double t, int flux,
                               const T* __restrict__ X, long long ldX, T* __restrict__ C, long long ldC)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (q >= np * 2 * nth) return;
    const long long P = q / (2 * nth);
    const double* tab = ctab + (cstart + P) * 5;
    const int n = cn[cstart + P];
    const T* x = X + (long long)b * ldX + xboff + q;
    const long long stride = np * 2 * nth;
    double acc = 0.0;
    for (int it = 0; it < n; ++it) {
        const double g = bmaux_weight(tab, it, t, flux);
        if (g != 0.0) acc += g * (double)x[it * stride];
    }
    C[(long long)b * ldC + cboff + q] = (T)acc;
}

// adX[b][xboff + ((it NP + P) nth + th) 2 + c] += g(it, P) adC[b][cboff + (P nth + th) 2 + c]
// for one frequency: one thread per coefficient of the frequency
template <typename T>
__global__ void k_bmaux_scatter(const double* __restrict__ ctab, const int32_t* __restrict__ cn, long long cstart,
                                long long np, int nth, int nit, long long xboff, long long cboff, double t, int flux,
                                const T* __restrict__ adC, long long ldC, T* __restrict__ adX, long long ldX)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    const long long per = np * 2 * nth;
    if (e >= per * nit) return;
    const int it = (int)(e / per);
    const long long q = e - (long long)it * per;
    const long long P = q / (2 * nth);
    if (it >= cn[cstart + P]) return;                 // padded time centre: weight 0
    const double g = bmaux_weight(ctab + (cstart + P) * 5, it, t, flux);
    if (g == 0.0) return;
    T* a = adX + (long long)b * ldX + xboff + e;
    *a = (T)((double)*a + g * (double)adC[(long long)b * ldC + cboff + q]);
}

}  // namespace vd

namespace {

struct BmTables {
    std::vector<int32_t> row_freq, row_pat, row_n, fx_i, tx_ptr, tx_x, tx_e, pat_cbase, fy_j, ty_ptr, ty_y, ty_e,
        freq_rowoff;
    std::vector<long long> row_cb, freq_boff, freq_np;
    std::vector<double> fx_c, fx_s, fy_c, fy_s;
};

// Lattice rows share x patterns: same centres, same cos(lat), same frequency.
struct PatState {
    std::map<std::vector<double>, int> pat_of;
    std::vector<std::vector<std::vector<std::pair<int, double>>>> pat_cols;   // [pat][x] -> (i, xx)
    std::vector<int> pat_n, pat_freq;
};

void add_row(vd_bm_plan* p, BmTables& tb, PatState& ps, int iff, double la, double cl,
             const std::vector<double>& lons, const std::vector<double>& xc, double k2, long long& cb)
{
    BmFreq& F = p->fr[iff];
    const int nx = (int)xc.size();
    std::vector<double> key = lons;
    key.push_back(cl);
    key.push_back((double)iff);
    int pat;
    auto it = ps.pat_of.find(key);
    if (it != ps.pat_of.end()) {
        pat = it->second;
    } else {
        pat = (int)ps.pat_cols.size();
        ps.pat_of[key] = pat;
        std::vector<std::vector<std::pair<int, double>>> cols((size_t)nx);
        for (int x = 0; x < nx; ++x)
            for (int i = 0; i < (int)lons.size(); ++i) {
                const double xx = (xc[x] - lons[i]) / k2 * cl;
                if (std::fabs(xx) <= F.DX) cols[x].push_back({i, xx});
            }
        ps.pat_cols.push_back(std::move(cols));
        ps.pat_n.push_back((int)lons.size());
        ps.pat_freq.push_back(iff);
    }
    tb.row_freq.push_back(iff);
    tb.row_pat.push_back(pat);
    tb.row_n.push_back((int)lons.size());
    tb.row_cb.push_back(cb);
    F.row_lons.push_back(lons);
    for (double lo : lons) {
        F.enslat.push_back(la);
        F.enslon.push_back(lo);
    }
    cb += (long long)lons.size();
}

// x tables (ELL per pattern and column, CSR per centre) and y tables (ELL per
// frequency and row, CSR per lattice row), with the per-direction cos / sin
// factors of the angle-sum split (sqrt(2) folded into y).
void build_xy(vd_bm_plan* p, BmTables& tb, const PatState& ps, const std::vector<double>& yc, double k2, int ny,
              int nx)
{
    const std::vector<double>& th = p->theta;
    int KX = 1;
    for (auto& pc : ps.pat_cols)
        for (auto& col : pc) KX = std::max(KX, (int)col.size());
    p->KX = KX;
    const int P = (int)ps.pat_cols.size(), nth = p->nth;
    tb.fx_i.assign((size_t)P * nx * KX, -1);
    tb.fx_c.assign((size_t)P * nth * nx * KX, 0.0);
    tb.fx_s.assign((size_t)P * nth * nx * KX, 0.0);
    tb.tx_ptr.push_back(0);
    for (int pt = 0; pt < P; ++pt) {
        const BmFreq& F = p->fr[ps.pat_freq[pt]];
        tb.pat_cbase.push_back((int)tb.tx_ptr.size() - 1);
        std::vector<std::vector<std::pair<int, int>>> by_centre((size_t)ps.pat_n[pt]);
        for (int x = 0; x < nx; ++x) {
            const auto& col = ps.pat_cols[pt][x];
            for (size_t e = 0; e < col.size(); ++e) {
                const double xx = col[e].second;
                const double wx = mywindow(xx / F.DX);
                tb.fx_i[((size_t)pt * nx + x) * KX + e] = col[e].first;
                for (int t = 0; t < nth; ++t) {
                    const double kx = F.k * std::cos(th[t]);
                    const size_t w = (((size_t)pt * nth + t) * nx + x) * KX + e;
                    tb.fx_c[w] = wx * std::cos(kx * xx);
                    tb.fx_s[w] = wx * std::sin(kx * xx);
                }
                by_centre[col[e].first].push_back({x, (int)e});
            }
        }
        for (auto& lst : by_centre) {
            for (auto& pr : lst) {
                tb.tx_x.push_back(pr.first);
                tb.tx_e.push_back(pr.second);
            }
            tb.tx_ptr.push_back((int32_t)tb.tx_x.size());
        }
    }
    std::vector<std::vector<std::vector<std::pair<int, double>>>> ycols((size_t)p->nf);
    int KY = 1;
    for (int iff = 0; iff < p->nf; ++iff) {
        const BmFreq& F = p->fr[iff];
        ycols[iff].resize((size_t)ny);
        for (int y = 0; y < ny; ++y)
            for (int j = 0; j < (int)F.rows_lat.size(); ++j) {
                const double yy = (yc[y] - F.rows_lat[j]) / k2;
                if (std::fabs(yy) <= F.DX) ycols[iff][y].push_back({j, yy});
            }
        for (auto& l : ycols[iff]) KY = std::max(KY, (int)l.size());
    }
    p->KY = KY;
    tb.fy_j.assign((size_t)p->nf * ny * KY, -1);
    tb.fy_c.assign((size_t)p->nf * nth * ny * KY, 0.0);
    tb.fy_s.assign((size_t)p->nf * nth * ny * KY, 0.0);
    tb.ty_ptr.push_back(0);
    for (int iff = 0; iff < p->nf; ++iff) {
        const BmFreq& F = p->fr[iff];
        std::vector<std::vector<std::pair<int, int>>> by_row(F.rows_lat.size());
        for (int y = 0; y < ny; ++y) {
            const auto& l = ycols[iff][y];
            for (size_t e = 0; e < l.size(); ++e) {
                const double yy = l[e].second;
                const double wy = std::sqrt(2.0) * mywindow(yy / F.DX);
                tb.fy_j[((size_t)iff * ny + y) * KY + e] = l[e].first;
                for (int t = 0; t < nth; ++t) {
                    const double ky = F.k * std::sin(th[t]);
                    const size_t w = (((size_t)iff * nth + t) * ny + y) * KY + e;
                    tb.fy_c[w] = wy * std::cos(ky * yy);
                    tb.fy_s[w] = wy * std::sin(ky * yy);
                }
                by_row[l[e].first].push_back({y, (int)e});
            }
        }
        for (auto& lst : by_row) {
            for (auto& pr : lst) {
                tb.ty_y.push_back(pr.first);
                tb.ty_e.push_back(pr.second);
            }
            tb.ty_ptr.push_back((int32_t)tb.ty_y.size());
        }
    }
}

// active (time centre, weight) lists per (basis time, frequency), padded to NA
void pack_time(vd_bm_plan* p, const std::vector<std::vector<std::pair<int, double>>>& act)
{
    int NA = 1;
    for (auto& l : act) NA = std::max(NA, (int)l.size());
    p->NA = NA;
    p->tact_n.assign((size_t)p->ntime * p->nf, 0);
    p->tact_it.assign((size_t)p->ntime * p->nf * NA, 0);
    p->tact_g.assign((size_t)p->ntime * p->nf * NA, 0.0);
    for (size_t s = 0; s < act.size(); ++s) {
        p->tact_n[s] = (int)act[s].size();
        for (size_t a = 0; a < act[s].size(); ++a) {
            p->tact_it[s * NA + a] = act[s][a].first;
            p->tact_g[s * NA + a] = act[s][a].second;
        }
    }
}

int bm_build(vd_bm_plan* p, const vd_basis_grid* g, BmTables& tb)
{
    const vd_bm_params& q = p->prm;
    const int ny = g->ny, nx = g->nx;
    const bool geo = g->geographic != 0;
    const double k2 = geo ? 1.0 / 110 : 1.0;
    std::vector<double> xc(g->xc_host, g->xc_host + nx), yc(g->yc_host, g->yc_host + ny);
    for (double v : xc) if (!std::isfinite(v)) return VD_ERR_ARG;
    for (double v : yc) if (!std::isfinite(v)) return VD_ERR_ARG;
    if (!(q.npsp > 0) || !(q.facpsp > 0) || !(q.lmin > 0) || !(q.lmax > q.lmin) || !(q.facns > 0) ||
        !(q.facnlt > 0) || !(q.tdecmin > 0) || !(q.tdecmax >= q.tdecmin))
        return VD_ERR_ARG;
    const double LON_MIN = *std::min_element(xc.begin(), xc.end());
    double LON_MAX = *std::max_element(xc.begin(), xc.end());
    const double LAT_MIN = *std::min_element(yc.begin(), yc.end());
    const double LAT_MAX = *std::max_element(yc.begin(), yc.end());
    if (LON_MAX < LON_MIN) LON_MAX += 360.;
    p->times.assign(g->time_host, g->time_host + g->ntime);
    const double deltat = *std::max_element(p->times.begin(), p->times.end()) -
                          *std::min_element(p->times.begin(), p->times.end());
    auto cosd = [&](double lat) { return geo ? std::cos(lat * M_PI / 180.) : 1.0; };
    auto window = [&](double x) { return q.flux ? mywindow_flux(x) : mywindow(x); };
    std::vector<int8_t> land;
    bool any_land = false;
    if (g->land_host) {
        land.assign(g->land_host, g->land_host + (size_t)ny * nx);
        for (int8_t v : land) any_land |= (v != 0);
    }

    // frequencies and directions (basis.py:577-587)
    const double lstep = std::log(1 + q.facpsp / q.npsp);
    std::vector<double> logff = np_arange(std::log(1. / q.lmin), std::log(1. / q.lmax) - lstep, -lstep);
    std::reverse(logff.begin(), logff.end());
    if (logff.size() < 2) return VD_ERR_ARG;
    std::vector<double> ff(logff.size());
    for (size_t i = 0; i < ff.size(); ++i) ff[i] = std::exp(logff[i]);
    const double dff0 = ff[1] - ff[0];
    std::vector<double> th = np_linspace(0, M_PI, (int)(M_PI * ff[0] / dff0 * q.facpsp));
    if (th.size() < 2) return VD_ERR_ARG;
    th.pop_back();
    p->theta = th;
    p->nth = (int)th.size();
    p->nf = (int)ff.size();
    p->fr.resize(ff.size());

    // lattices, time centres, Q (basis.py:603-690)
    PatState ps;
    long long boff = 0;
    int rowoff = 0;
    for (int iff = 0; iff < p->nf; ++iff) {
        BmFreq& F = p->fr[iff];
        F.ff = ff[iff];
        F.k = 2 * M_PI * ff[iff];
        F.DX = 1. / ff[iff] * q.npsp * 0.5;
        F.DXG = F.DX / q.facns;
        const double dlat = F.DXG * k2;
        const double lat0 = LAT_MIN - pymod(LAT_MIN, dlat) - F.DX * k2;
        const double lat1 = LAT_MAX + F.DX * k2 * 1.5;
        F.rows_lat = np_arange(lat0, lat1, dlat);
        F.rowoff = rowoff;
        F.boff = boff;
        long long cb = 0;
        for (double la : F.rows_lat) {
            const double cl = cosd(la);
            const double dlon = F.DXG / cl * k2;
            const double lon0 = LON_MIN - pymod(LON_MIN, dlon) - F.DX / cl * k2;
            const double lon1 = LON_MAX + F.DX / cl * k2 * 1.5;
            std::vector<double> lons0 = np_arange(lon0, lon1, dlon), lons;
            for (double lo : lons0) {
                if (any_land) {
                    // keep a centre only if its box of radius 1/ff holds an unmasked point (basis.py:632-645)
                    bool keep = false;
                    for (int yy = 0; yy < ny && !keep; ++yy) {
                        if (!(std::fabs((yc[yy] - la) / k2) <= 1. / ff[iff])) continue;
                        for (int xx = 0; xx < nx; ++xx)
                            if (std::fabs((xc[xx] - lo) / k2 * cl) <= 1. / ff[iff] && !land[(size_t)yy * nx + xx]) {
                                keep = true;
                                break;
                            }
                    }
                    if (!keep) continue;
                }
                lons.push_back(lo);
            }
            add_row(p, tb, ps, iff, la, cl, lons, xc, k2, cb);
        }
        F.NP = cb;
        double td = q.tmeso * std::pow(q.lmeso, q.sloptdec) * std::pow(ff[iff], q.sloptdec);
        td *= q.factdec;
        if (td < q.tdecmin) td = q.tdecmin;
        if (td > q.tdecmax) td = q.tdecmax;
        F.tdec = td;
        const double t0 = pymod(-q.time_ref, td);
        F.enst = np_arange(t0 - td / q.facnlt, deltat + td / q.facnlt, td / q.facnlt);
        F.norm_fact = window_norm(td, window);
        F.Q = (1 / ff[iff] > q.lmeso) ? q.Qmax / q.facns
                                      : q.Qmax / q.facns * std::pow(q.lmeso, q.slopQ) * std::pow(ff[iff], q.slopQ);
        boff += (long long)F.enst.size() * 2 * p->nth * F.NP;
        rowoff += (int)F.rows_lat.size();
        tb.freq_rowoff.push_back(F.rowoff);
        tb.freq_boff.push_back(F.boff);
        tb.freq_np.push_back(F.NP);
    }
    p->nbasis = boff;
    p->R = rowoff;
    build_xy(p, tb, ps, yc, k2, ny, nx);

    // time weights of the JAX form: |dt| <= tdec (basis.py:1026-1035)
    std::vector<std::vector<std::pair<int, double>>> act((size_t)p->ntime * p->nf);
    for (int kt = 0; kt < p->ntime; ++kt)
        for (int iff = 0; iff < p->nf; ++iff) {
            const BmFreq& F = p->fr[iff];
            auto& lst = act[(size_t)kt * p->nf + iff];
            for (int it = 0; it < (int)F.enst.size(); ++it) {
                const double dt = p->times[kt] - F.enst[it];
                if (!(std::fabs(dt) > F.tdec || std::isnan(F.enst[it]))) {
                    double fact = window(dt / F.tdec);
                    if (q.norm_time) fact /= F.norm_fact;
                    lst.push_back({it, fact});
                }
            }
        }
    pack_time(p, act);
    return VD_OK;
}

// Orthogonal multilinear interpolation of an auxiliary field [f][lat][lon]
// at (f, la, lo), NaN outside the coordinates (xarray's DataArray.interp with
// 1-D indexers, linear); a NaN corner gives NaN.
double aux_value(const vd_bm_plan* p, const std::vector<double>& fld, double f, double la, double lo)
{
    auto bracket = [](const std::vector<double>& c, double x, int& i0, double& w) {
        const int n = (int)c.size();
        if (!(x >= c[0] && x <= c[n - 1])) return false;
        int i = (int)(std::upper_bound(c.begin(), c.end(), x) - c.begin()) - 1;
        i = std::min(std::max(i, 0), n - 2);
        i0 = i;
        w = (x - c[i]) / (c[i + 1] - c[i]);
        return true;
    };
    int a, b, c;
    double wa, wb, wc;
    if (!bracket(p->ax_f, f, a, wa) || !bracket(p->ax_lat, la, b, wb) || !bracket(p->ax_lon, lo, c, wc))
        return std::nan("");
    const size_t NL = p->ax_lat.size(), NO = p->ax_lon.size();
    auto at = [&](int i, int j, int k) { return fld[((size_t)i * NL + j) * NO + k]; };
    // along f, then lat, then lon, as the successive 1-D interpolations do
    double v[2][2];
    for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k) v[j][k] = (1 - wa) * at(a, b + j, c + k) + wa * at(a + 1, b + j, c + k);
    const double v0 = (1 - wb) * v[0][0] + wb * v[1][0], v1 = (1 - wb) * v[0][1] + wb * v[1][1];
    return (1 - wc) * v0 + wc * v1;
}

// nanmean of a field over the 10 x 10 grid of a centre's box of half-width DX
// (basis.py:2005-2009, 2066-2072); NaN when every value is NaN
double aux_box_mean(const vd_bm_plan* p, const std::vector<double>& fld, double f, double la, double lo,
                    double dlat, double dlon)
{
    const std::vector<double> elon = np_linspace(lo - dlon, lo + dlon, 10), elat = np_linspace(la - dlat, la + dlat, 10);
    double sum = 0.0;
    int cnt = 0;
    for (double y : elat)
        for (double x : elon) {
            const double v = aux_value(p, fld, f, y, x);
            if (!std::isnan(v)) {
                sum += v;
                ++cnt;
            }
        }
    return cnt ? sum / cnt : std::nan("");
}

// Basis_bmaux (basis.py:1741-2393): the wave-packet lattice ending at
// LAT_MAX + DX and LON_MAX + DX/cos (1947-1954), per-centre times and Q
int bmaux_build(vd_bm_plan* p, const vd_basis_grid* g, BmTables& tb)
{
    const vd_bmaux_params& q = p->aprm;
    const int ny = g->ny, nx = g->nx;
    const bool geo = g->geographic != 0;
    const double k2 = geo ? 1.0 / 110 : 1.0;
    std::vector<double> xc(g->xc_host, g->xc_host + nx), yc(g->yc_host, g->yc_host + ny);
    for (double v : xc) if (!std::isfinite(v)) return VD_ERR_ARG;
    for (double v : yc) if (!std::isfinite(v)) return VD_ERR_ARG;
    if (!(q.npsp > 0) || !(q.facpsp > 0) || !(q.lmin > 0) || !(q.lmax > q.lmin) || !(q.facns > 0) ||
        !(q.facnlt > 0) || !(q.tdecmin > 0) || !(q.tdecmax >= q.tdecmin))
        return VD_ERR_ARG;
    const double LON_MIN = *std::min_element(xc.begin(), xc.end());
    double LON_MAX = *std::max_element(xc.begin(), xc.end());
    const double LAT_MIN = *std::min_element(yc.begin(), yc.end());
    const double LAT_MAX = *std::max_element(yc.begin(), yc.end());
    if (LON_MAX < LON_MIN) LON_MAX += 360.;
    p->times.assign(g->time_host, g->time_host + g->ntime);
    const double deltat = *std::max_element(p->times.begin(), p->times.end()) -
                          *std::min_element(p->times.begin(), p->times.end());
    auto cosd = [&](double lat) { return geo ? std::cos(lat * M_PI / 180.) : 1.0; };
    auto window = [&](double x) { return q.flux ? mywindow_flux(x) : mywindow(x); };
    std::vector<int8_t> land;
    bool any_land = false;
    if (g->land_host) {
        land.assign(g->land_host, g->land_host + (size_t)ny * nx);
        for (int8_t v : land) any_land |= (v != 0);
    }
    const double lstep = std::log(1 + q.facpsp / q.npsp);
    std::vector<double> logff = np_arange(std::log(1. / q.lmin), std::log(1. / q.lmax) - lstep, -lstep);
    std::reverse(logff.begin(), logff.end());
    if (logff.size() < 2) return VD_ERR_ARG;
    std::vector<double> ff(logff.size());
    for (size_t i = 0; i < ff.size(); ++i) ff[i] = std::exp(logff[i]);
    std::vector<double> th = np_linspace(0, M_PI, (int)(M_PI * ff[0] / (ff[1] - ff[0]) * q.facpsp));
    if (th.size() < 2) return VD_ERR_ARG;
    th.pop_back();
    p->theta = th;
    p->nth = (int)th.size();
    p->nf = (int)ff.size();
    p->fr.resize(ff.size());
    PatState ps;
    long long boff = 0, cboff = 0, cstart = 0;
    int rowoff = 0;
    for (int iff = 0; iff < p->nf; ++iff) {
        BmFreq& F = p->fr[iff];
        F.ff = ff[iff];
        F.k = 2 * M_PI * ff[iff];
        F.DX = 1. / ff[iff] * q.npsp * 0.5;
        F.DXG = F.DX / q.facns;
        const double dlat = F.DXG * k2;
        const double lat0 = LAT_MIN - pymod(LAT_MIN, dlat) - F.DX * k2;
        const double lat1 = LAT_MAX + F.DX * k2;
        F.rows_lat = np_arange(lat0, lat1, dlat);
        F.rowoff = rowoff;
        long long cb = 0;
        for (double la : F.rows_lat) {
            const double cl = cosd(la);
            const double dlon = F.DXG / cl * k2;
            const double lon0 = LON_MIN - pymod(LON_MIN, dlon) - F.DX / cl * k2;
            const double lon1 = LON_MAX + F.DX / cl * k2;
            std::vector<double> lons0 = np_arange(lon0, lon1, dlon), lons;
            for (double lo : lons0) {
                if (any_land) {
                    bool keep = false;
                    for (int yy = 0; yy < ny && !keep; ++yy) {
                        if (!(std::fabs((yc[yy] - la) / k2) <= 1. / ff[iff])) continue;
                        for (int xx = 0; xx < nx; ++xx)
                            if (std::fabs((xc[xx] - lo) / k2 * cl) <= 1. / ff[iff] && !land[(size_t)yy * nx + xx]) {
                                keep = true;
                                break;
                            }
                    }
                    if (!keep) continue;
                }
                lons.push_back(lo);
            }
            add_row(p, tb, ps, iff, la, cl, lons, xc, k2, cb);
        }
        F.NP = cb;
        // per-centre decorrelation time, window integral, time centres and std
        int nit = 0;
        for (long long P = 0; P < F.NP; ++P) {
            const double la = F.enslat[P], lo = F.enslon[P];
            const double bdlon = F.DX * k2 / cosd(la), bdlat = F.DX * k2;
            const double m = aux_box_mean(p, p->ax_td, ff[iff], la, lo, bdlat, bdlon);
            double td = std::isnan(m) ? 0.0 : m;
            td *= q.factdec;
            if (td < q.tdecmin) td = q.tdecmin;
            if (td > q.tdecmax) td = q.tdecmax;
            const double nrm = q.norm_time ? window_norm(td, window) : 1.0;
            const double t0 = pymod(-q.time_ref, td);
            const double step = td / q.facnlt, start = t0 - step;
            const std::vector<double> en = np_arange(start, deltat + step, step);
            const double sd = aux_box_mean(p, p->ax_sd, ff[iff], la, lo, bdlat, bdlon);
            F.c_tdec.push_back(td);
            F.c_norm.push_back(nrm);
            F.c_start.push_back(start);
            F.c_step.push_back(step);
            F.c_delta.push_back((start + step) - start);
            F.c_n.push_back((int)en.size());
            F.c_std.push_back(std::isnan(sd) ? 1e-10 : sd);
            nit = std::max(nit, (int)en.size());
        }
        F.nit = nit;
        F.tdec = 0.0;
        F.enst.assign((size_t)nit, std::nan(""));
        F.boff = boff;
        F.cboff = cboff;
        F.cstart = cstart;
        boff += (long long)nit * 2 * p->nth * F.NP;
        cboff += 2LL * p->nth * F.NP;
        cstart += F.NP;
        rowoff += (int)F.rows_lat.size();
        tb.freq_rowoff.push_back(F.rowoff);
        tb.freq_boff.push_back(F.cboff);     // the passes read the time-reduced coefficients
        tb.freq_np.push_back(F.NP);
    }
    p->nbasis = boff;
    p->cbasis = cboff;
    p->ncentres = cstart;
    p->R = rowoff;
    build_xy(p, tb, ps, yc, k2, ny, nx);
    // the passes run on the time-reduced coefficients: one "time centre" of weight 1
    std::vector<std::vector<std::pair<int, double>>> act((size_t)p->ntime * p->nf, {{0, 1.0}});
    pack_time(p, act);
    return VD_OK;
}

// Gaspari-Cohn function of mapping/src/tools.py:16-46 for one value
double gaspari_cohn(double r, double c)
{
    if (c <= 0) return 0.0;
    const double ra = 2 * std::fabs(r) / c;
    if (ra <= 1.)
        return -0.25 * std::pow(ra, 5) + 0.5 * std::pow(ra, 4) + 0.625 * std::pow(ra, 3) - 5. / 3. * (ra * ra) + 1.;
    if (ra > 1. && ra <= 2.)
        return 1. / 12. * std::pow(ra, 5) - 0.5 * std::pow(ra, 4) + 0.625 * std::pow(ra, 3) + 5. / 3. * (ra * ra) -
               5. * ra + 4. - 2. / 3. / ra;
    return 0.0;
}

// np.arange(c, lo, -step)[::-1] followed by np.arange(c, hi, step)[1:]
std::vector<double> centred_axis(double c, double lo, double hi, double step)
{
    std::vector<double> a = np_arange(c, lo, -step);
    std::reverse(a.begin(), a.end());
    std::vector<double> b = np_arange(c, hi, step);
    for (size_t i = 1; i < b.size(); ++i) a.push_back(b[i]);
    return a;
}

// Basis_wavelet3d.set_basis (basis.py:2684-2843)
int wav_build(vd_bm_plan* p, const vd_basis_grid* g, BmTables& tb)
{
    const vd_wavelet_params& q = p->wprm;
    const int ny = g->ny, nx = g->nx;
    const bool geo = g->geographic != 0;
    const double k2 = geo ? 1.0 / 110 : 1.0;
    std::vector<double> xc(g->xc_host, g->xc_host + nx), yc(g->yc_host, g->yc_host + ny);
    for (double v : xc) if (!std::isfinite(v)) return VD_ERR_ARG;
    for (double v : yc) if (!std::isfinite(v)) return VD_ERR_ARG;
    if (!(q.npsp > 0) || !(q.facpsp > 0) || !(q.lmin > 0) || !(q.lmax > q.lmin) || !(q.facnst > 0) ||
        !(q.tmin > 0) || !(q.tmax > q.tmin))
        return VD_ERR_ARG;
    const double LON_MIN = *std::min_element(xc.begin(), xc.end());
    double LON_MAX = *std::max_element(xc.begin(), xc.end());
    const double LAT_MIN = *std::min_element(yc.begin(), yc.end());
    const double LAT_MAX = *std::max_element(yc.begin(), yc.end());
    if (LON_MAX < LON_MIN) LON_MAX += 360.;
    p->times.assign(g->time_host, g->time_host + g->ntime);
    const double TIME_MIN = *std::min_element(p->times.begin(), p->times.end());
    const double TIME_MAX = *std::max_element(p->times.begin(), p->times.end());
    auto cosd = [&](double lat) { return geo ? std::cos(lat * M_PI / 180.) : 1.0; };
    std::vector<int8_t> land;
    bool any_land = false;
    if (g->land_host) {
        land.assign(g->land_host, g->land_host + (size_t)ny * nx);
        for (int8_t v : land) any_land |= (v != 0);
    }
    // pseudo-frequencies in space and time, directions (2689-2715)
    const double lstep = std::log(1 + q.facpsp / q.npsp);
    auto freqs = [&](double lo, double hi) {
        std::vector<double> l = np_arange(std::log(1. / lo), std::log(1. / hi) - lstep, -lstep);
        std::reverse(l.begin(), l.end());
        std::vector<double> f;
        for (double v : l) {
            const double e = std::exp(v);
            if (1. / e <= hi) f.push_back(e);
        }
        return f;
    };
    std::vector<double> fs = freqs(q.lmin, q.lmax), ft = freqs(q.tmin, q.tmax);
    if (fs.size() < 2 || ft.empty()) return VD_ERR_ARG;
    std::vector<double> th = np_linspace(0, M_PI, (int)(M_PI * fs[0] / (fs[1] - fs[0]) * q.facpsp));
    if (th.size() < 2) return VD_ERR_ARG;
    th.pop_back();
    p->theta = th;
    p->nth = (int)th.size();
    p->nf = (int)fs.size();
    p->fr.resize(fs.size());
    // time centres of every time frequency, shared by all space frequencies (2773-2796)
    std::vector<double> enst, tscale, tnorm;
    for (double f : ft) {
        const double DXt = 1. / f * q.npsp * 0.5;
        std::vector<double> e = centred_axis((TIME_MIN + TIME_MAX) / 2, TIME_MIN - DXt, TIME_MAX + DXt, DXt / q.facnst);
        // norm_fact: running integral of the window on linspace(-DXt, DXt) (50 points), its maximum
        std::vector<double> tt = np_linspace(-DXt, DXt, 50);
        double acc = 0, mx = 0;
        for (size_t i = 0; i + 1 < tt.size(); ++i) {
            acc = acc + gaspari_cohn(tt[i], DXt) * (tt[i + 1] - tt[i]);
            mx = std::max(mx, acc);
        }
        for (double c : e) {
            enst.push_back(c);
            tscale.push_back(DXt);
            tnorm.push_back(mx);
        }
    }
    // space lattices (2717-2771)
    PatState ps;
    long long boff = 0;
    int rowoff = 0;
    for (int iff = 0; iff < p->nf; ++iff) {
        BmFreq& F = p->fr[iff];
        F.ff = fs[iff];
        F.k = 2 * M_PI * fs[iff];
        F.DX = 1. / fs[iff] * q.npsp * 0.5;
        F.DXG = F.DX / q.facnst;
        F.rows_lat = centred_axis((LAT_MIN + LAT_MAX) / 2, LAT_MIN - F.DX * k2, LAT_MAX + F.DX * k2, F.DXG * k2);
        F.rowoff = rowoff;
        F.boff = boff;
        long long cb = 0;
        std::vector<double> kept_lat;
        for (double la : F.rows_lat) {
            const double cl = cosd(la);
            std::vector<double> lons0 = centred_axis((LON_MIN + LON_MAX) / 2, LON_MIN - F.DX / cl * k2,
                                                     LON_MAX + F.DX / cl * k2, F.DXG / cl * k2),
                                lons;
            for (double lo : lons0) {
                if (any_land) {
                    // drop a centre whose box of half-width 0.5/fs holds only masked points (2752-2764)
                    bool keep = false;
                    for (int yy = 0; yy < ny && !keep; ++yy) {
                        if (!(std::fabs((yc[yy] - la) / k2) <= .5 / fs[iff])) continue;
                        for (int xx = 0; xx < nx; ++xx)
                            if (std::fabs((xc[xx] - lo) / k2 * cl) <= .5 / fs[iff] && !land[(size_t)yy * nx + xx]) {
                                keep = true;
                                break;
                            }
                    }
                    if (!keep) continue;
                }
                lons.push_back(lo);
            }
            add_row(p, tb, ps, iff, la, cl, lons, xc, k2, cb);
        }
        F.NP = cb;
        F.enst = enst;
        F.tscale = tscale;
        F.tnorm = tnorm;
        F.tdec = tscale.empty() ? 0.0 : tscale[0];
        F.Q = q.sigma_Q;
        boff += (long long)enst.size() * 2 * p->nth * F.NP;
        rowoff += (int)F.rows_lat.size();
        tb.freq_rowoff.push_back(F.rowoff);
        tb.freq_boff.push_back(F.boff);
        tb.freq_np.push_back(F.NP);
    }
    p->nbasis = boff;
    p->R = rowoff;
    build_xy(p, tb, ps, yc, k2, ny, nx);
    // time weights (2902-2922): |dt| < DXt, Gaspari-Cohn / norm_fact, kept when non-zero
    std::vector<std::vector<std::pair<int, double>>> act((size_t)p->ntime * p->nf);
    for (int kt = 0; kt < p->ntime; ++kt)
        for (int iff = 0; iff < p->nf; ++iff) {
            const BmFreq& F = p->fr[iff];
            auto& lst = act[(size_t)kt * p->nf + iff];
            for (int it = 0; it < (int)F.enst.size(); ++it) {
                const double dt = p->times[kt] - F.enst[it];
                if (std::fabs(dt) < F.tscale[it]) {
                    const double fact = gaspari_cohn(dt, F.tscale[it]) / F.tnorm[it];
                    if (fact != 0) lst.push_back({it, fact});
                }
            }
        }
    pack_time(p, act);
    return VD_OK;
}

template <typename T>
int bm_upload(vd_bm_plan* p, const BmTables& tb, const int8_t* land_host)
{
    Packer pk;
    const size_t o_rf = pk.add(tb.row_freq), o_rp = pk.add(tb.row_pat), o_rn = pk.add(tb.row_n),
                 o_fxi = pk.add(tb.fx_i), o_txp = pk.add(tb.tx_ptr), o_txx = pk.add(tb.tx_x),
                 o_txe = pk.add(tb.tx_e), o_pcb = pk.add(tb.pat_cbase), o_fyj = pk.add(tb.fy_j),
                 o_typ = pk.add(tb.ty_ptr), o_tyy = pk.add(tb.ty_y), o_tye = pk.add(tb.ty_e),
                 o_fro = pk.add(tb.freq_rowoff), o_tn = pk.add(p->tact_n), o_tit = pk.add(p->tact_it),
                 o_rcb = pk.add(tb.row_cb), o_fbo = pk.add(tb.freq_boff), o_fnp = pk.add(tb.freq_np),
                 o_fxc = pk.add_as<T>(tb.fx_c), o_fxs = pk.add_as<T>(tb.fx_s), o_fyc = pk.add_as<T>(tb.fy_c),
                 o_fys = pk.add_as<T>(tb.fy_s), o_tg = pk.add_as<T>(p->tact_g);
    size_t o_land = 0;
    bool any_land = false;
    std::vector<int8_t> land;
    if (land_host) {
        land.assign(land_host, land_host + (size_t)p->ny * p->nx);
        for (int8_t v : land) any_land |= (v != 0);
        if (any_land) o_land = pk.add(land);
    }
    VD_CUDA_TRY(cudaMalloc(&p->dev, pk.blob.size()));
    VD_CUDA_TRY(cudaMemcpy(p->dev, pk.blob.data(), pk.blob.size(), cudaMemcpyHostToDevice));
    unsigned char* b = (unsigned char*)p->dev;
    p->row_freq = (const int32_t*)(b + o_rf);
    p->row_pat = (const int32_t*)(b + o_rp);
    p->row_n = (const int32_t*)(b + o_rn);
    p->fx_i = (const int32_t*)(b + o_fxi);
    p->tx_ptr = (const int32_t*)(b + o_txp);
    p->tx_x = (const int32_t*)(b + o_txx);
    p->tx_e = (const int32_t*)(b + o_txe);
    p->pat_cbase = (const int32_t*)(b + o_pcb);
    p->fy_j = (const int32_t*)(b + o_fyj);
    p->ty_ptr = (const int32_t*)(b + o_typ);
    p->ty_y = (const int32_t*)(b + o_tyy);
    p->ty_e = (const int32_t*)(b + o_tye);
    p->freq_rowoff = (const int32_t*)(b + o_fro);
    p->d_tact_n = (const int32_t*)(b + o_tn);
    p->d_tact_it = (const int32_t*)(b + o_tit);
    p->row_cb = (const long long*)(b + o_rcb);
    p->freq_boff = (const long long*)(b + o_fbo);
    p->freq_np = (const long long*)(b + o_fnp);
    p->fx_c = b + o_fxc;
    p->fx_s = b + o_fxs;
    p->fy_c = b + o_fyc;
    p->fy_s = b + o_fys;
    p->d_tact_g = b + o_tg;
    p->land = any_land ? (const int8_t*)(b + o_land) : nullptr;
    if (p->kind == 2 && p->ncentres > 0) {
        std::vector<double> tab;
        std::vector<int32_t> cn;
        tab.reserve((size_t)p->ncentres * 5);
        for (const BmFreq& F : p->fr)
            for (long long P = 0; P < F.NP; ++P) {
                tab.insert(tab.end(), {F.c_tdec[P], F.c_norm[P], F.c_start[P], F.c_step[P], F.c_delta[P]});
                cn.push_back(F.c_n[P]);
            }
        Packer pa;
        const size_t o_tab = pa.add(tab), o_cn = pa.add(cn);
        VD_CUDA_TRY(cudaMalloc(&p->dev_aux, pa.blob.size()));
        VD_CUDA_TRY(cudaMemcpy(p->dev_aux, pa.blob.data(), pa.blob.size(), cudaMemcpyHostToDevice));
        p->d_ctab = (const double*)((unsigned char*)p->dev_aux + o_tab);
        p->d_cn = (const int32_t*)((unsigned char*)p->dev_aux + o_cn);
    }
    return VD_OK;
}

size_t bm_ws_bytes(const vd_bm_plan* p, int batch)
{
    const size_t es = p->dtype == VD_F64 ? 8 : 4;
    const size_t rows = (size_t)batch * p->R * p->nth * 2 * p->nx * es;
    if (p->kind != 2) return rows;
    return ((rows + 255) & ~size_t(255)) + (size_t)batch * p->cbasis * es;
}

// time-reduced coefficients of the auxiliary-field basis (behind the rows)
template <typename T>
T* bmaux_coeffs(const vd_bm_plan* p, int B, T* ws)
{
    const size_t rows = (size_t)B * p->R * p->nth * 2 * p->nx * sizeof(T);
    return (T*)((char*)ws + ((rows + 255) & ~size_t(255)));
}

template <typename T>
int bm_project(const vd_bm_plan* p, int B, int k, const T* X, long long ldX, T* phi, int acc, T* ws,
               cudaStream_t st)
{
    const vd::BmDev<T> d = vd::bm_view<T>(p);
    const unsigned gx = (unsigned)((p->nx + 127) / 128);
    if (p->kind == 2) {
        T* C = bmaux_coeffs<T>(p, B, ws);
        for (const BmFreq& F : p->fr) {
            const long long n = F.NP * 2 * p->nth;
            if (n == 0) continue;
            vd::k_bmaux_reduce<T><<<dim3((unsigned)((n + 127) / 128), B), 128, 0, st>>>(
                p->d_ctab, p->d_cn, F.cstart, F.NP, p->nth, F.boff, F.cboff, p->times[k], p->aprm.flux, X, ldX, C,
                p->cbasis);
            VD_LAUNCH_CHECK();
        }
        X = C;
        ldX = p->cbasis;
        k = 0;
    }
    vd::k_bm_xpass<T><<<dim3(gx, p->R * p->nth, B), 128, 0, st>>>(d, k, X, ldX, ws);
    VD_LAUNCH_CHECK();
    vd::k_bm_ypass<T><<<dim3(gx, p->ny, B), 128, 0, st>>>(d, ws, phi, acc);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int bm_project_T(const vd_bm_plan* p, int B, int k, const T* adphi, T* adX, long long ldX, T* ws, cudaStream_t st)
{
    const vd::BmDev<T> d = vd::bm_view<T>(p);
    const unsigned gx = (unsigned)((p->nx + 127) / 128);
    vd::k_bmT_ypass<T><<<dim3(gx, p->R * p->nth, B), 128, 0, st>>>(d, adphi, ws);
    VD_LAUNCH_CHECK();
    if (p->kind != 2) {
        vd::k_bmT_xpass<T><<<dim3(p->R, B), 128, 0, st>>>(d, k, ws, adX, ldX);
        VD_LAUNCH_CHECK();
        return VD_OK;
    }
    T* C = bmaux_coeffs<T>(p, B, ws);
    VD_CUDA_TRY(cudaMemsetAsync(C, 0, (size_t)B * p->cbasis * sizeof(T), st));
    vd::k_bmT_xpass<T><<<dim3(p->R, B), 128, 0, st>>>(d, 0, ws, C, p->cbasis);
    VD_LAUNCH_CHECK();
    for (const BmFreq& F : p->fr) {
        const long long n = (long long)F.nit * F.NP * 2 * p->nth;
        if (n == 0) continue;
        vd::k_bmaux_scatter<T><<<dim3((unsigned)((n + 127) / 128), B), 128, 0, st>>>(
            p->d_ctab, p->d_cn, F.cstart, F.NP, p->nth, F.nit, F.boff, F.cboff, p->times[k], p->aprm.flux, C,
            p->cbasis, adX, ldX);
        VD_LAUNCH_CHECK();
    }
    return VD_OK;
}

int bm_check(const vd_bm_plan* p, int B, int k, long long ldX, const void* a, const void* b, void* ws, size_t wsb)
{
    if (!p || p->host_only || !p->dev) return VD_ERR_ARG;
    if (B < 1 || B > 65535 || k < 0 || k >= p->ntime || !a || !b || !ws) return VD_ERR_ARG;
    if (B > 1 && ldX < p->nbasis) return VD_ERR_ARG;
    if (wsb < bm_ws_bytes(p, B)) return VD_ERR_WORKSPACE;
    return VD_OK;
}

}  // namespace

static vd_status bm_create(vd_bm_plan** out, const vd_basis_grid* g, const vd_bm_params* prm,
                           const vd_wavelet_params* wprm, const vd_bmaux_params* aprm = nullptr)
{
    if (!out || !g || (!prm && !wprm && !aprm)) return VD_ERR_ARG;
    *out = nullptr;
    if (g->ny < 1 || g->nx < 1 || !g->xc_host || !g->yc_host || g->ntime < 1 || !g->time_host) return VD_ERR_ARG;
    if (g->dtype != VD_F32 && g->dtype != VD_F64) return VD_ERR_ARG;
    for (int i = 0; i < g->ntime; ++i)
        if (!std::isfinite(g->time_host[i])) return VD_ERR_ARG;
    vd_bm_plan* p = new (std::nothrow) vd_bm_plan();
    if (!p) return VD_ERR_ARG;
    p->ny = g->ny; p->nx = g->nx; p->dtype = g->dtype; p->geographic = g->geographic;
    p->host_only = g->host_only; p->ntime = g->ntime;
    if (prm) p->prm = *prm;
    if (wprm) {
        p->kind = 1;
        p->wprm = *wprm;
    }
    if (aprm) {
        p->kind = 2;
        p->aprm = *aprm;
        const vd_bmaux_params& a = *aprm;
        if (a.aux_nf < 2 || a.aux_nlat < 2 || a.aux_nlon < 2 || !a.aux_f || !a.aux_lat || !a.aux_lon ||
            !a.aux_tdec || !a.aux_std) {
            delete p;
            return VD_ERR_ARG;
        }
        const size_t n = (size_t)a.aux_nf * a.aux_nlat * a.aux_nlon;
        p->ax_f.assign(a.aux_f, a.aux_f + a.aux_nf);
        p->ax_lat.assign(a.aux_lat, a.aux_lat + a.aux_nlat);
        p->ax_lon.assign(a.aux_lon, a.aux_lon + a.aux_nlon);
        p->ax_td.assign(a.aux_tdec, a.aux_tdec + n);
        p->ax_sd.assign(a.aux_std, a.aux_std + n);
        p->aprm.aux_f = p->aprm.aux_lat = p->aprm.aux_lon = p->aprm.aux_tdec = p->aprm.aux_std = nullptr;
        for (const std::vector<double>* c : {&p->ax_f, &p->ax_lat, &p->ax_lon})
            for (size_t i = 1; i < c->size(); ++i)
                if (!((*c)[i] > (*c)[i - 1])) {
                    delete p;
                    return VD_ERR_ARG;
                }
    }
    BmTables tb;
    int st = p->kind == 1 ? wav_build(p, g, tb) : (p->kind == 2 ? bmaux_build(p, g, tb) : bm_build(p, g, tb));
    if (st == VD_OK && ((long long)p->R * p->nth > 65535 || p->ny > 65535 || p->R > 65535)) st = VD_ERR_UNSUPPORTED;
    if (st == VD_OK && !p->host_only)
        st = p->dtype == VD_F64 ? bm_upload<double>(p, tb, g->land_host) : bm_upload<float>(p, tb, g->land_host);
    if (st != VD_OK) {
        if (p->dev) cudaFree(p->dev);
        if (p->dev_aux) cudaFree(p->dev_aux);
        delete p;
        return st;
    }
    *out = p;
    return VD_OK;
}

extern "C" vd_status vd_bmaux_plan_create(vd_bm_plan** out, const vd_basis_grid* g, const vd_bmaux_params* prm)
{
    return prm ? bm_create(out, g, nullptr, nullptr, prm) : VD_ERR_ARG;
}

extern "C" vd_status vd_bmaux_centres(const vd_bm_plan* p, int iff, double* tdec, double* norm, int* nt)
{
    if (!p || p->kind != 2 || iff < 0 || iff >= p->nf) return VD_ERR_ARG;
    const BmFreq& F = p->fr[iff];
    if (tdec) std::copy(F.c_tdec.begin(), F.c_tdec.end(), tdec);
    if (norm) std::copy(F.c_norm.begin(), F.c_norm.end(), norm);
    if (nt) std::copy(F.c_n.begin(), F.c_n.end(), nt);
    return VD_OK;
}

extern "C" vd_status vd_bm_plan_create(vd_bm_plan** out, const vd_basis_grid* g, const vd_bm_params* prm)
{
    return prm ? bm_create(out, g, prm, nullptr) : VD_ERR_ARG;
}

extern "C" vd_status vd_wavelet_plan_create(vd_bm_plan** out, const vd_basis_grid* g, const vd_wavelet_params* prm)
{
    return prm ? bm_create(out, g, nullptr, prm) : VD_ERR_ARG;
}

extern "C" vd_status vd_bm_plan_destroy(vd_bm_plan* p)
{
    if (!p) return VD_ERR_ARG;
    if (p->dev) cudaFree(p->dev);
    if (p->dev_aux) cudaFree(p->dev_aux);
    delete p;
    return VD_OK;
}

extern "C" long long vd_bm_nbasis(const vd_bm_plan* p) { return p ? p->nbasis : 0; }

extern "C" vd_status vd_bm_shape(const vd_bm_plan* p, int* nf, int* ntheta, double* theta_host)
{
    if (!p) return VD_ERR_ARG;
    if (nf) *nf = p->nf;
    if (ntheta) *ntheta = p->nth;
    if (theta_host) std::copy(p->theta.begin(), p->theta.end(), theta_host);
    return VD_OK;
}

extern "C" vd_status vd_bm_frequency(const vd_bm_plan* p, int iff, double* ff, double* tdec, long long* offset,
                                     int* ntime_centres, int* nspace_centres)
{
    if (!p || iff < 0 || iff >= p->nf) return VD_ERR_ARG;
    const BmFreq& F = p->fr[iff];
    if (ff) *ff = F.ff;
    if (tdec) *tdec = F.tdec;
    if (offset) *offset = F.boff;
    if (ntime_centres) *ntime_centres = (int)F.enst.size();
    if (nspace_centres) *nspace_centres = (int)F.NP;
    return VD_OK;
}

extern "C" vd_status vd_bm_lattice(const vd_bm_plan* p, int iff, double* enst, double* enslat, double* enslon)
{
    if (!p || iff < 0 || iff >= p->nf) return VD_ERR_ARG;
    const BmFreq& F = p->fr[iff];
    if (enst && p->kind == 2) {
        // [NP][nit], NaN beyond a centre's own count (basis.py:2029-2035)
        for (long long P = 0; P < F.NP; ++P)
            for (int it = 0; it < F.nit; ++it)
                enst[P * F.nit + it] = it >= F.c_n[P] ? std::nan("")
                                       : it == 0 ? F.c_start[P]
                                       : it == 1 ? F.c_start[P] + F.c_step[P]
                                                 : F.c_start[P] + (double)it * F.c_delta[P];
    } else if (enst) {
        std::copy(F.enst.begin(), F.enst.end(), enst);
    }
    if (enslat) std::copy(F.enslat.begin(), F.enslat.end(), enslat);
    if (enslon) std::copy(F.enslon.begin(), F.enslon.end(), enslon);
    return VD_OK;
}

extern "C" vd_status vd_bm_q(const vd_bm_plan* p, double* q)
{
    if (!p || !q) return VD_ERR_ARG;
    if (p->kind == 2) {
        for (const BmFreq& F : p->fr)
            for (int it = 0; it < F.nit; ++it)
                for (long long P = 0; P < F.NP; ++P) {
                    const double v = (it < F.c_n[P] ? F.c_std[P] : 1e-10) * p->aprm.facQ;
                    std::fill(q + F.boff + (it * F.NP + P) * 2 * p->nth,
                              q + F.boff + (it * F.NP + P + 1) * 2 * p->nth, v);
                }
        return VD_OK;
    }
    for (const BmFreq& F : p->fr) {
        const long long n = (long long)F.enst.size() * 2 * p->nth * F.NP;
        std::fill(q + F.boff, q + F.boff + n, F.Q);
    }
    return VD_OK;
}

extern "C" vd_status vd_bm_time_weights(const vd_bm_plan* p, int k, int iff, int* count, int* it, double* w)
{
    if (!p || !count || k < 0 || k >= p->ntime || iff < 0 || iff >= p->nf) return VD_ERR_ARG;
    if (p->kind == 2) return VD_ERR_UNSUPPORTED;      // per-centre time weights
    const size_t s = (size_t)k * p->nf + iff;
    *count = p->tact_n[s];
    for (int a = 0; a < p->tact_n[s]; ++a) {
        if (it) it[a] = p->tact_it[s * p->NA + a];
        if (w) w[a] = p->tact_g[s * p->NA + a];
    }
    return VD_OK;
}

extern "C" size_t vd_bm_workspace_bytes(const vd_bm_plan* p, int batch)
{
    if (!p || batch < 1) return 0;
    return bm_ws_bytes(p, batch);
}

extern "C" vd_status vd_bm_project(const vd_bm_plan* p, int B, int k, const void* X, long long ldX, void* phi,
                                   int accumulate, void* ws, size_t wsb, void* stream)
{
    const int st = bm_check(p, B, k, ldX, X, phi, ws, wsb);
    if (st != VD_OK) return st;
    if (p->dtype == VD_F64)
        return bm_project<double>(p, B, k, (const double*)X, ldX, (double*)phi, accumulate, (double*)ws,
                                  (cudaStream_t)stream);
    return bm_project<float>(p, B, k, (const float*)X, ldX, (float*)phi, accumulate, (float*)ws,
                             (cudaStream_t)stream);
}

extern "C" vd_status vd_bm_project_T(const vd_bm_plan* p, int B, int k, const void* adphi, void* adX,
                                     long long ldX, void* ws, size_t wsb, void* stream)
{
    const int st = bm_check(p, B, k, ldX, adphi, adX, ws, wsb);
    if (st != VD_OK) return st;
    if (p->dtype == VD_F64)
        return bm_project_T<double>(p, B, k, (const double*)adphi, (double*)adX, ldX, (double*)ws,
                                    (cudaStream_t)stream);
    return bm_project_T<float>(p, B, k, (const float*)adphi, (float*)adX, ldX, (float*)ws, (cudaStream_t)stream);
}
