// Gaussian space-time reduced basis: phi = G(t) X and adX += G(t)^T adphi.
//
// Reference: mapping/src/basis.py, Basis_gauss3d (1170-1555) and Basis_multi
// (4039-4135). The reference stores each component's space part as a CSC
// matrix Gauss_xy [nphys x Nx] and its time part as one weight per
// (time centre, basis time); operg is Gauss_xy . (sum over active time
// centres of g_it X[it, :]).
//
// Here the grid is rectilinear (x/longitude per column, y/latitude per row),
// so every footprint factorises: a centre (row j of the lattice, centre i of
// that row) contributes wy_j(y) * wx_{j,i}(x) at grid point (y, x), where
// wy_j(y) = mywindow((y - lat_j)/km2deg / sigma_D) and wx the same in x with
// the cos(lat_j) stretch (basis.py:1403-1419). The product is then two banded
// passes instead of a sparse matrix:
//   x pass  T[r][x]  = sum_i wx_{r,i}(x) * (sum_a g_a X[it_a, cb_r + i])   (r: lattice row)
//   y pass  phi[y][x] = land ? 0 : sum_c sum_j wy_{c,j}(y) T[row(c, j)][x]
// and the transpose runs them backwards:
//   y^T     U[r][x]  = sum_y wy_r(y) * (land ? 0 : adphi[y][x])
//   x^T     adX[it_a, cb_r + i] += g_a * sum_x wx_{r,i}(x) U[r][x]
// Every output is written by one thread (no atomics): results are
// deterministic. Tables are built on the host in float64 with the
// reference's formulas (including NumPy's arange/linspace value sequences),
// so footprint membership and weights match the reference's CSC entries.
#include "vd_internal.cuh"
#include "vd_basis_host.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <tuple>
#include <vector>

namespace {

using namespace vd::basis_host;

struct HostComp {
    vd_gauss3d_params p;
    double norm_fact = 1.0;
    std::vector<double> enst;        // time centres
    std::vector<double> rows_lat;    // lattice rows (ENSLAT1)
    std::vector<int> row_n;          // centres per lattice row
    std::vector<long long> row_cb;   // first centre index of each row
    std::vector<double> enslat, enslon;
    long long Nx = 0;                // space centres
    long long boff = 0;              // offset of the component in X
    int rowoff = 0;                  // first global lattice row
    double window(double x) const { return p.flux ? mywindow_flux(x) : mywindow(x); }
};

}  // namespace

struct vd_basis_plan {
    int ny = 0, nx = 0, dtype = VD_F32, geographic = 0, host_only = 0;
    int ncomp = 0, ntime = 0;
    long long nbasis = 0;
    int R = 0;          // lattice rows over all components
    int KX = 0, KY = 0; // ELL widths of the x and y tables
    int NA = 0;         // max active time centres per (time, component)
    std::vector<HostComp> comps;
    std::vector<double> times;
    // time weights [ntime][ncomp][NA]
    std::vector<int> tact_n, tact_it;
    std::vector<double> tact_g;
    // device tables (one allocation)
    void* dev = nullptr;
    // pointers into dev
    const int32_t *row_comp, *row_pat, *row_n, *fx_i, *fy_j, *ty_ptr, *ty_row, *tx_ptr, *tx_col,
        *pat_cbase, *comp_rowoff, *d_tact_n, *d_tact_it;
    const long long *row_cb, *comp_boff, *comp_Nx;
    const void *fx_w, *fy_w, *ty_w, *tx_w, *d_tact_g;
    const int8_t* land;
};

namespace vd {

template <typename T>
struct BasisDev {
    int ny, nx, R, KX, KY, NA, ncomp;
    const int32_t *row_comp, *row_pat, *row_n, *fx_i, *fy_j, *ty_ptr, *ty_row, *tx_ptr, *tx_col,
        *pat_cbase, *comp_rowoff, *tact_n, *tact_it;
    const long long *row_cb, *comp_boff, *comp_Nx;
    const T *fx_w, *fy_w, *ty_w, *tx_w, *tact_g;
    const int8_t* land;
};

template <typename T>
BasisDev<T> dev_view(const vd_basis_plan* p)
{
    BasisDev<T> d;
    d.ny = p->ny; d.nx = p->nx; d.R = p->R; d.KX = p->KX; d.KY = p->KY; d.NA = p->NA;
    d.ncomp = p->ncomp;
    d.row_comp = p->row_comp; d.row_pat = p->row_pat; d.row_n = p->row_n;
    d.fx_i = p->fx_i; d.fy_j = p->fy_j; d.ty_ptr = p->ty_ptr; d.ty_row = p->ty_row;
    d.tx_ptr = p->tx_ptr; d.tx_col = p->tx_col; d.pat_cbase = p->pat_cbase;
    d.comp_rowoff = p->comp_rowoff; d.tact_n = p->d_tact_n; d.tact_it = p->d_tact_it;
    d.row_cb = p->row_cb; d.comp_boff = p->comp_boff; d.comp_Nx = p->comp_Nx;
    d.fx_w = (const T*)p->fx_w; d.fy_w = (const T*)p->fy_w; d.ty_w = (const T*)p->ty_w;
    d.tx_w = (const T*)p->tx_w; d.tact_g = (const T*)p->d_tact_g;
    d.land = p->land;
    return d;
}

// x pass of G: one thread per (lattice row r, column x, window b).
template <typename T>
__global__ void __launch_bounds__(128)
k_basis_xpass(BasisDev<T> d, int k, const T* __restrict__ X, long long ldX, T* __restrict__ Tw)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y, b = blockIdx.z;
    if (x >= d.nx) return;
    const int c = d.row_comp[r];
    const long long Nx = d.comp_Nx[c];
    const T* Xr = X + (long long)b * ldX + d.comp_boff[c] + d.row_cb[r];
    const int ta = (k * d.ncomp + c) * d.NA;
    const int na = d.tact_n[k * d.ncomp + c];
    const long long e0 = ((long long)d.row_pat[r] * d.nx + x) * d.KX;
    T acc = T(0);
    for (int e = 0; e < d.KX; ++e) {
        const int i = d.fx_i[e0 + e];
        if (i < 0) break;
        T z = T(0);
        for (int a = 0; a < na; ++a) z += d.tact_g[ta + a] * Xr[(long long)d.tact_it[ta + a] * Nx + i];
        acc += d.fx_w[e0 + e] * z;
    }
    Tw[((long long)b * d.R + r) * d.nx + x] = acc;
}

// y pass of G: one thread per (y, x, b), summing every component.
template <typename T>
__global__ void __launch_bounds__(128)
k_basis_ypass(BasisDev<T> d, const T* __restrict__ Tw, T* __restrict__ phi, int accumulate)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, b = blockIdx.z;
    if (x >= d.nx) return;
    T acc = T(0);
    for (int c = 0; c < d.ncomp; ++c) {
        const long long e0 = ((long long)c * d.ny + y) * d.KY;
        const T* Tc = Tw + ((long long)b * d.R + d.comp_rowoff[c]) * d.nx + x;
        for (int e = 0; e < d.KY; ++e) {
            const int j = d.fy_j[e0 + e];
            if (j < 0) break;
            acc += d.fy_w[e0 + e] * Tc[(long long)j * d.nx];
        }
    }
    const long long o = ((long long)b * d.ny + y) * d.nx + x;
    if (d.land && d.land[(long long)y * d.nx + x]) acc = T(0);
    phi[o] = accumulate ? phi[o] + acc : acc;
}

// y pass of G^T: one thread per (lattice row r, x, b).
template <typename T>
__global__ void __launch_bounds__(128)
k_basisT_ypass(BasisDev<T> d, const T* __restrict__ adphi, T* __restrict__ Uw)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y, b = blockIdx.z;
    if (x >= d.nx) return;
    const T* a = adphi + (long long)b * d.ny * d.nx + x;
    T acc = T(0);
    for (int e = d.ty_ptr[r]; e < d.ty_ptr[r + 1]; ++e) {
        const int y = d.ty_row[e];
        T v = a[(long long)y * d.nx];
        if (d.land && d.land[(long long)y * d.nx + x]) v = T(0);
        acc += d.ty_w[e] * v;
    }
    Uw[((long long)b * d.R + r) * d.nx + x] = acc;
}

// x pass of G^T: one CTA per (lattice row r, window b), one thread per centre.
template <typename T>
__global__ void __launch_bounds__(128)
k_basisT_xpass(BasisDev<T> d, int k, const T* __restrict__ Uw, T* __restrict__ adX, long long ldX)
{
    const int r = blockIdx.x, b = blockIdx.y;
    const int c = d.row_comp[r];
    const long long Nx = d.comp_Nx[c];
    const int ta = (k * d.ncomp + c) * d.NA;
    const int na = d.tact_n[k * d.ncomp + c];
    const T* U = Uw + ((long long)b * d.R + r) * d.nx;
    T* A = adX + (long long)b * ldX + d.comp_boff[c] + d.row_cb[r];
    const int base = d.pat_cbase[d.row_pat[r]];
    for (int i = threadIdx.x; i < d.row_n[r]; i += blockDim.x) {
        T s = T(0);
        for (int e = d.tx_ptr[base + i]; e < d.tx_ptr[base + i + 1]; ++e) s += d.tx_w[e] * U[d.tx_col[e]];
        for (int a = 0; a < na; ++a) {
            const long long o = (long long)d.tact_it[ta + a] * Nx + i;
            A[o] += d.tact_g[ta + a] * s;
        }
    }
}

}  // namespace vd

namespace {

struct Tables {
    std::vector<int32_t> row_comp, row_pat, row_n, fx_i, fy_j, ty_ptr, ty_row, tx_ptr, tx_col, pat_cbase,
        comp_rowoff;
    std::vector<long long> row_cb, comp_boff, comp_Nx;
    std::vector<double> fx_w, fy_w, ty_w, tx_w;
};

// Lattice, time weights and banded tables of every component.
int build_host(vd_basis_plan* p, const vd_basis_grid* g, const vd_gauss3d_params* cp, Tables& tb)
{
    const int ny = g->ny, nx = g->nx;
    const bool geo = g->geographic != 0;
    const double k = geo ? 1.0 / 110 : 1.0;
    std::vector<double> xc(g->xc_host, g->xc_host + nx), yc(g->yc_host, g->yc_host + ny);
    for (double v : xc) if (!std::isfinite(v)) return VD_ERR_ARG;
    for (double v : yc) if (!std::isfinite(v)) return VD_ERR_ARG;
    const double LON_MIN = *std::min_element(xc.begin(), xc.end());
    double LON_MAX = *std::max_element(xc.begin(), xc.end());
    const double LAT_MIN = *std::min_element(yc.begin(), yc.end());
    const double LAT_MAX = *std::max_element(yc.begin(), yc.end());
    if (LON_MAX < LON_MIN) LON_MAX += 360.;
    p->times.assign(g->time_host, g->time_host + g->ntime);
    const double TMIN = *std::min_element(p->times.begin(), p->times.end());
    const double TMAX = *std::max_element(p->times.begin(), p->times.end());
    auto cosd = [&](double lat) { return geo ? std::cos(lat * M_PI / 180.) : 1.0; };
    auto wrap = [&](double d) { return geo ? pymod(d + 180, 360) - 180 : d; };

    // x-pattern dedup: rows of one component with the same lattice share tables
    std::map<std::tuple<int, double, double, long, double>, int> pat_of;
    std::vector<std::vector<std::vector<std::pair<int, double>>>> pat_cols;  // [pat][x] -> (i, w)
    std::vector<int> pat_n;

    long long boff = 0;
    int rowoff = 0;
    p->comps.resize(p->ncomp);
    for (int c = 0; c < p->ncomp; ++c) {
        HostComp& hc = p->comps[c];
        hc.p = cp[c];
        const vd_gauss3d_params& q = cp[c];
        if (!(q.sigma_D > 0) || !(q.sigma_T > 0) || !(q.facns > 0) || !(q.facnlt > 0)) return VD_ERR_ARG;
        if (q.has_time_spinup && !(q.time_spinup != 0)) return VD_ERR_ARG;
        if (q.normalize_fact) {                                   // basis.py:1278-1283
            const int num = 50;
            const double step = (q.sigma_T - (-q.sigma_T)) / (num - 1);
            double tt[num], tmp = 0.0, mx = 0.0;
            for (int i = 0; i < num; ++i) tt[i] = (double)i * step + (-q.sigma_T);
            tt[num - 1] = q.sigma_T;
            for (int i = 0; i < num - 1; ++i) {
                tmp = tmp + hc.window(tt[i] / q.sigma_T) * (tt[i + 1] - tt[i]);
                mx = std::max(mx, tmp);
            }
            hc.norm_fact = mx;
        }
        // space lattice (basis.py:1303-1316)
        const double dlat = q.sigma_D / q.facns * k;
        const double lat0 = LAT_MIN - pymod(LAT_MIN, dlat) - q.sigma_D * (1 - 1. / q.facns) * k;
        const double lat1 = LAT_MAX + 1.5 * dlat;
        hc.rows_lat = np_arange(lat0, lat1, dlat);
        hc.rowoff = rowoff;
        hc.boff = boff;
        long long cb = 0;
        for (double la : hc.rows_lat) {
            const double cl = cosd(la);
            const double dlon = q.sigma_D / q.facns / cl * k;
            const double lon0 = LON_MIN - pymod(LON_MIN, dlon) - q.sigma_D * (1 - 1. / q.facns) / cl * k;
            const double lon1 = LON_MAX + dlon * 1.5;
            std::vector<double> lons = np_arange(lon0, lon1, dlon);
            const int n = (int)lons.size();
            auto key = std::make_tuple(c, lon0, dlon, (long)n, cl);
            int pat;
            auto it = pat_of.find(key);
            if (it != pat_of.end()) {
                pat = it->second;
            } else {
                pat = (int)pat_cols.size();
                pat_of[key] = pat;
                std::vector<std::vector<std::pair<int, double>>> cols((size_t)nx);
                for (int x = 0; x < nx; ++x)
                    for (int i = 0; i < n; ++i) {
                        const double xx = wrap(xc[x] - lons[i]) / k * cl;
                        if (std::fabs(xx) <= q.sigma_D) cols[x].push_back({i, mywindow(xx / q.sigma_D)});
                    }
                pat_cols.push_back(std::move(cols));
                pat_n.push_back(n);
            }
            tb.row_comp.push_back(c);
            tb.row_pat.push_back(pat);
            tb.row_n.push_back(n);
            tb.row_cb.push_back(cb);
            hc.row_n.push_back(n);
            hc.row_cb.push_back(cb);
            for (double lo : lons) {
                hc.enslat.push_back(la);
                hc.enslon.push_back(lo);
            }
            cb += n;
        }
        hc.Nx = cb;
        // time lattice (basis.py:1320-1321)
        hc.enst = np_arange(-q.sigma_T * (1 - 1. / q.facnlt), (TMAX - TMIN) + 1.5 * q.sigma_T / q.facnlt,
                            q.sigma_T / q.facnlt);
        boff += (long long)hc.enst.size() * hc.Nx;
        rowoff += (int)hc.rows_lat.size();
        tb.comp_rowoff.push_back(hc.rowoff);
        tb.comp_boff.push_back(hc.boff);
        tb.comp_Nx.push_back(hc.Nx);
    }
    p->nbasis = boff;
    p->R = rowoff;

    // x tables (ELL per pattern column, CSR per pattern centre)
    int KX = 1;
    for (auto& pc : pat_cols)
        for (auto& col : pc) KX = std::max(KX, (int)col.size());
    p->KX = KX;
    const int P = (int)pat_cols.size();
    tb.fx_i.assign((size_t)P * nx * KX, -1);
    tb.fx_w.assign((size_t)P * nx * KX, 0.0);
    tb.tx_ptr.push_back(0);
    for (int pt = 0; pt < P; ++pt) {
        tb.pat_cbase.push_back((int)tb.tx_ptr.size() - 1);
        std::vector<std::vector<std::pair<int, double>>> by_centre((size_t)pat_n[pt]);
        for (int x = 0; x < nx; ++x) {
            const auto& col = pat_cols[pt][x];
            for (size_t e = 0; e < col.size(); ++e) {
                tb.fx_i[((size_t)pt * nx + x) * KX + e] = col[e].first;
                tb.fx_w[((size_t)pt * nx + x) * KX + e] = col[e].second;
                by_centre[col[e].first].push_back({x, col[e].second});
            }
        }
        for (auto& lst : by_centre) {
            for (auto& pr : lst) {
                tb.tx_col.push_back(pr.first);
                tb.tx_w.push_back(pr.second);
            }
            tb.tx_ptr.push_back((int32_t)tb.tx_col.size());
        }
    }

    // y tables (ELL per component row, CSR per lattice row)
    std::vector<std::vector<std::vector<std::pair<int, double>>>> ycols((size_t)p->ncomp);
    int KY = 1;
    for (int c = 0; c < p->ncomp; ++c) {
        const HostComp& hc = p->comps[c];
        ycols[c].resize((size_t)ny);
        for (int y = 0; y < ny; ++y)
            for (int j = 0; j < (int)hc.rows_lat.size(); ++j) {
                const double yy = (yc[y] - hc.rows_lat[j]) / k;
                if (std::fabs(yy) <= hc.p.sigma_D) ycols[c][y].push_back({j, mywindow(yy / hc.p.sigma_D)});
            }
        for (auto& l : ycols[c]) KY = std::max(KY, (int)l.size());
    }
    p->KY = KY;
    tb.fy_j.assign((size_t)p->ncomp * ny * KY, -1);
    tb.fy_w.assign((size_t)p->ncomp * ny * KY, 0.0);
    tb.ty_ptr.push_back(0);
    for (int c = 0; c < p->ncomp; ++c) {
        const int nr = (int)p->comps[c].rows_lat.size();
        std::vector<std::vector<std::pair<int, double>>> by_row((size_t)nr);
        for (int y = 0; y < ny; ++y) {
            const auto& l = ycols[c][y];
            for (size_t e = 0; e < l.size(); ++e) {
                tb.fy_j[((size_t)c * ny + y) * KY + e] = l[e].first;
                tb.fy_w[((size_t)c * ny + y) * KY + e] = l[e].second;
                by_row[l[e].first].push_back({y, l[e].second});
            }
        }
        for (auto& lst : by_row) {
            for (auto& pr : lst) {
                tb.ty_row.push_back(pr.first);
                tb.ty_w.push_back(pr.second);
            }
            tb.ty_ptr.push_back((int32_t)tb.ty_row.size());
        }
    }

    // time weights per (basis time, component) (basis.py:1423-1446)
    std::vector<std::vector<std::pair<int, double>>> act((size_t)p->ntime * p->ncomp);
    int NA = 1;
    for (int kt = 0; kt < p->ntime; ++kt) {
        const double t = p->times[kt];
        for (int c = 0; c < p->ncomp; ++c) {
            const HostComp& hc = p->comps[c];
            auto& lst = act[(size_t)kt * p->ncomp + c];
            for (int it = 0; it < (int)hc.enst.size(); ++it) {
                const double dt = t - hc.enst[it];
                if (std::fabs(dt) < hc.p.sigma_T) {
                    double fact = hc.window(dt / hc.p.sigma_T);
                    if (hc.p.normalize_fact) fact /= hc.norm_fact;
                    if (hc.p.has_time_spinup && t < hc.p.time_spinup)
                        fact *= (1 - hc.window(t / hc.p.time_spinup));
                    if (fact != 0) lst.push_back({it, fact});
                }
            }
            NA = std::max(NA, (int)lst.size());
        }
    }
    p->NA = NA;
    p->tact_n.assign((size_t)p->ntime * p->ncomp, 0);
    p->tact_it.assign((size_t)p->ntime * p->ncomp * NA, 0);
    p->tact_g.assign((size_t)p->ntime * p->ncomp * NA, 0.0);
    for (size_t s = 0; s < act.size(); ++s) {
        p->tact_n[s] = (int)act[s].size();
        for (size_t a = 0; a < act[s].size(); ++a) {
            p->tact_it[s * NA + a] = act[s][a].first;
            p->tact_g[s * NA + a] = act[s][a].second;
        }
    }
    return VD_OK;
}

template <typename T>
int upload(vd_basis_plan* p, const Tables& tb, const int8_t* land_host)
{
    Packer pk;
    const size_t o_row_comp = pk.add(tb.row_comp), o_row_pat = pk.add(tb.row_pat), o_row_n = pk.add(tb.row_n),
                 o_fx_i = pk.add(tb.fx_i), o_fy_j = pk.add(tb.fy_j), o_ty_ptr = pk.add(tb.ty_ptr),
                 o_ty_row = pk.add(tb.ty_row), o_tx_ptr = pk.add(tb.tx_ptr), o_tx_col = pk.add(tb.tx_col),
                 o_pat_cbase = pk.add(tb.pat_cbase), o_comp_rowoff = pk.add(tb.comp_rowoff),
                 o_tact_n = pk.add(p->tact_n), o_tact_it = pk.add(p->tact_it), o_row_cb = pk.add(tb.row_cb),
                 o_comp_boff = pk.add(tb.comp_boff), o_comp_Nx = pk.add(tb.comp_Nx),
                 o_fx_w = pk.add_as<T>(tb.fx_w), o_fy_w = pk.add_as<T>(tb.fy_w), o_ty_w = pk.add_as<T>(tb.ty_w),
                 o_tx_w = pk.add_as<T>(tb.tx_w), o_tact_g = pk.add_as<T>(p->tact_g);
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
    p->row_comp = (const int32_t*)(b + o_row_comp);
    p->row_pat = (const int32_t*)(b + o_row_pat);
    p->row_n = (const int32_t*)(b + o_row_n);
    p->fx_i = (const int32_t*)(b + o_fx_i);
    p->fy_j = (const int32_t*)(b + o_fy_j);
    p->ty_ptr = (const int32_t*)(b + o_ty_ptr);
    p->ty_row = (const int32_t*)(b + o_ty_row);
    p->tx_ptr = (const int32_t*)(b + o_tx_ptr);
    p->tx_col = (const int32_t*)(b + o_tx_col);
    p->pat_cbase = (const int32_t*)(b + o_pat_cbase);
    p->comp_rowoff = (const int32_t*)(b + o_comp_rowoff);
    p->d_tact_n = (const int32_t*)(b + o_tact_n);
    p->d_tact_it = (const int32_t*)(b + o_tact_it);
    p->row_cb = (const long long*)(b + o_row_cb);
    p->comp_boff = (const long long*)(b + o_comp_boff);
    p->comp_Nx = (const long long*)(b + o_comp_Nx);
    p->fx_w = b + o_fx_w;
    p->fy_w = b + o_fy_w;
    p->ty_w = b + o_ty_w;
    p->tx_w = b + o_tx_w;
    p->d_tact_g = b + o_tact_g;
    p->land = any_land ? (const int8_t*)(b + o_land) : nullptr;
    return VD_OK;
}

size_t ws_bytes(const vd_basis_plan* p, int batch)
{
    return (size_t)batch * p->R * p->nx * (p->dtype == VD_F64 ? 8 : 4);
}

}  // namespace

extern "C" vd_status vd_basis_plan_create(vd_basis_plan** out, const vd_basis_grid* g, int ncomp,
                                          const vd_gauss3d_params* comps)
{
    if (!out || !g || !comps || ncomp < 1) return VD_ERR_ARG;
    *out = nullptr;
    if (g->ny < 1 || g->nx < 1 || !g->xc_host || !g->yc_host || g->ntime < 1 || !g->time_host) return VD_ERR_ARG;
    if (g->dtype != VD_F32 && g->dtype != VD_F64) return VD_ERR_ARG;
    for (int i = 0; i < g->ntime; ++i)
        if (!std::isfinite(g->time_host[i])) return VD_ERR_ARG;
    vd_basis_plan* p = new (std::nothrow) vd_basis_plan();
    if (!p) return VD_ERR_ARG;
    p->ny = g->ny; p->nx = g->nx; p->dtype = g->dtype; p->geographic = g->geographic;
    p->host_only = g->host_only; p->ncomp = ncomp; p->ntime = g->ntime;
    Tables tb;
    int st = build_host(p, g, comps, tb);
    if (st == VD_OK && (p->R > 65535 || p->ny > 65535)) st = VD_ERR_UNSUPPORTED;
    if (st == VD_OK && !p->host_only)
        st = p->dtype == VD_F64 ? upload<double>(p, tb, g->land_host) : upload<float>(p, tb, g->land_host);
    if (st != VD_OK) {
        if (p->dev) cudaFree(p->dev);
        delete p;
        return st;
    }
    *out = p;
    return VD_OK;
}

extern "C" vd_status vd_basis_plan_destroy(vd_basis_plan* p)
{
    if (!p) return VD_ERR_ARG;
    if (p->dev) cudaFree(p->dev);
    delete p;
    return VD_OK;
}

extern "C" long long vd_basis_nbasis(const vd_basis_plan* p) { return p ? p->nbasis : 0; }

extern "C" vd_status vd_basis_component(const vd_basis_plan* p, int c, long long* offset, int* nt, int* ns)
{
    if (!p || c < 0 || c >= p->ncomp) return VD_ERR_ARG;
    if (offset) *offset = p->comps[c].boff;
    if (nt) *nt = (int)p->comps[c].enst.size();
    if (ns) *ns = (int)p->comps[c].Nx;
    return VD_OK;
}

extern "C" vd_status vd_basis_lattice(const vd_basis_plan* p, int c, double* enst, double* enslat, double* enslon)
{
    if (!p || c < 0 || c >= p->ncomp) return VD_ERR_ARG;
    const HostComp& hc = p->comps[c];
    if (enst) std::copy(hc.enst.begin(), hc.enst.end(), enst);
    if (enslat) std::copy(hc.enslat.begin(), hc.enslat.end(), enslat);
    if (enslon) std::copy(hc.enslon.begin(), hc.enslon.end(), enslon);
    return VD_OK;
}

extern "C" vd_status vd_basis_q(const vd_basis_plan* p, double* q)
{
    if (!p || !q) return VD_ERR_ARG;
    for (const HostComp& hc : p->comps) {
        const double v = hc.p.sigma_Q / std::sqrt(hc.p.facns * hc.p.facnlt);
        std::fill(q + hc.boff, q + hc.boff + (long long)hc.enst.size() * hc.Nx, v);
    }
    return VD_OK;
}

extern "C" vd_status vd_basis_time_weights(const vd_basis_plan* p, int k, int c, int* count, int* it, double* w)
{
    if (!p || !count || k < 0 || k >= p->ntime || c < 0 || c >= p->ncomp) return VD_ERR_ARG;
    const size_t s = (size_t)k * p->ncomp + c;
    *count = p->tact_n[s];
    for (int a = 0; a < p->tact_n[s]; ++a) {
        if (it) it[a] = p->tact_it[s * p->NA + a];
        if (w) w[a] = p->tact_g[s * p->NA + a];
    }
    return VD_OK;
}

extern "C" size_t vd_basis_workspace_bytes(const vd_basis_plan* p, int batch)
{
    if (!p || batch < 1) return 0;
    return ws_bytes(p, batch);
}

namespace {

template <typename T>
int project(const vd_basis_plan* p, int B, int k, const T* X, long long ldX, T* phi, int acc, T* ws,
            cudaStream_t st)
{
    const vd::BasisDev<T> d = vd::dev_view<T>(p);
    const unsigned gx = (unsigned)((p->nx + 127) / 128);
    vd::k_basis_xpass<T><<<dim3(gx, p->R, B), 128, 0, st>>>(d, k, X, ldX, ws);
    VD_LAUNCH_CHECK();
    vd::k_basis_ypass<T><<<dim3(gx, p->ny, B), 128, 0, st>>>(d, ws, phi, acc);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int project_T(const vd_basis_plan* p, int B, int k, const T* adphi, T* adX, long long ldX, T* ws,
              cudaStream_t st)
{
    const vd::BasisDev<T> d = vd::dev_view<T>(p);
    const unsigned gx = (unsigned)((p->nx + 127) / 128);
    vd::k_basisT_ypass<T><<<dim3(gx, p->R, B), 128, 0, st>>>(d, adphi, ws);
    VD_LAUNCH_CHECK();
    vd::k_basisT_xpass<T><<<dim3(p->R, B), 128, 0, st>>>(d, k, ws, adX, ldX);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

int check_call(const vd_basis_plan* p, int B, int k, long long ldX, const void* a, const void* b, void* ws,
               size_t wsb)
{
    if (!p || p->host_only || !p->dev) return VD_ERR_ARG;
    if (B < 1 || B > 65535 || k < 0 || k >= p->ntime || !a || !b || !ws) return VD_ERR_ARG;
    if (B > 1 && ldX < p->nbasis) return VD_ERR_ARG;
    if (wsb < ws_bytes(p, B)) return VD_ERR_WORKSPACE;
    return VD_OK;
}

}  // namespace

extern "C" vd_status vd_basis_project(const vd_basis_plan* p, int B, int k, const void* X, long long ldX,
                                      void* phi, int accumulate, void* ws, size_t wsb, void* stream)
{
    const int st = check_call(p, B, k, ldX, X, phi, ws, wsb);
    if (st != VD_OK) return st;
    if (p->dtype == VD_F64)
        return project<double>(p, B, k, (const double*)X, ldX, (double*)phi, accumulate, (double*)ws,
                               (cudaStream_t)stream);
    return project<float>(p, B, k, (const float*)X, ldX, (float*)phi, accumulate, (float*)ws,
                          (cudaStream_t)stream);
}

extern "C" vd_status vd_basis_project_T(const vd_basis_plan* p, int B, int k, const void* adphi, void* adX,
                                        long long ldX, void* ws, size_t wsb, void* stream)
{
    const int st = check_call(p, B, k, ldX, adphi, adX, ws, wsb);
    if (st != VD_OK) return st;
    if (p->dtype == VD_F64)
        return project_T<double>(p, B, k, (const double*)adphi, (double*)adX, ldX, (double*)ws,
                                 (cudaStream_t)stream);
    return project_T<float>(p, B, k, (const float*)adphi, (float*)adX, ldX, (float*)ws, (cudaStream_t)stream);
}
