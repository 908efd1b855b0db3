"""Along-track observation operator for batches of assimilation windows.

Mirrors ``Obsop_interp_l3_jax`` (mapping/src/obsop.py:375-678):

- operator construction once per window set, as the reference does in
  ``process_obs``/``_sparse_op`` (obsop.py:417-460, 486-604): the ``npix``
  nearest grid points, neighbours beyond ``dmax`` (obsop.py:406) dropped,
  Gaussian weights exp(-d^2/(2(dmax/2)^2)) normalised per observation. The
  neighbour search and the weights run on the GPU (vd_obs_knn, a scan of the
  dmax disc: exactly the valid neighbours of a k-nearest search);
  ``build='host'`` uses a KDTree on the host instead. Synthetic Cartesian
  grids use planar km coordinates where the reference uses 3-D Cartesian km
  from lon/lat;
- misfit ``inverr*(Hx - y)`` with NaN -> 0 (obsop.py:610-628) and its adjoint
  (obsop.py:630-678) as GPU kernels (vd_obs_misfit / vd_obs_adjoint).

Storage on the device: observations of all windows sorted by (model step,
window); per observation four (grid index, weight) pairs with index -1 for
unused slots; for the adjoint, a CSR list per step of the touched (window,
grid point) pairs, so that the transpose is a deterministic gather.
"""
import ctypes

import numpy as np
import torch
from scipy.spatial import cKDTree

from . import _lib


def dmax_km(dx, dy, npix):
    """obsop.py:406 for uniform spacing dx, dy [m]."""
    return npix * np.sqrt(dx ** 2 + dy ** 2) * 1e-3 * np.sqrt(2) / 2


def l3_exclusion(ny, nx, mask=None, mask_borders=False):
    """[ny * nx] uint8 table of the grid points the scipy operator
    ``Obsop_interp_l3`` never weights (obsop.py:118-134, used at 207-211).

    - ``mask_borders``: the outer ring of the grid (obsop.py:126-134 match
      coordinates against the ring's; on a uniform grid that is the ring).
    - ``mask`` (True on land): the reference stores ``np.where(mask)[1]``,
      the column numbers of the masked points, and compares them with flat
      grid indices, so what it removes is the points of row 0 whose column
      holds a masked point. That rule is kept here as the reference applies
      it."""
    ex = np.zeros((ny, nx), dtype=np.uint8)
    if mask_borders:
        ex[0, :] = ex[-1, :] = 1
        ex[:, 0] = ex[:, -1] = 1
    flat = ex.reshape(-1)
    if mask is not None:
        cols = np.unique(np.where(np.asarray(mask, dtype=bool))[1])
        flat[cols] = 1
    return flat


def interp_rows(x_km, y_km, ny, nx, dx, dy, npix=4, exclude=None):
    """(idx [n, npix] with -1 for dropped neighbours, w [n, npix]) on a
    uniform grid whose point (0, 0) sits at (0 km, 0 km). ``exclude`` (an
    :func:`l3_exclusion` table) applies the scipy operator's rule: an excluded
    point keeps its place among the ``npix`` nearest and gets no weight."""
    gx, gy = np.meshgrid(np.arange(nx) * dx / 1e3, np.arange(ny) * dy / 1e3)
    tree = cKDTree(np.column_stack((gx.ravel(), gy.ravel())))
    D, ind = tree.query(np.column_stack((x_km, y_km)), k=npix)
    if npix == 1:
        D, ind = D[:, None], ind[:, None]
    dmax = dmax_km(dx, dy, npix)
    valid = D <= dmax
    if exclude is not None:
        valid &= np.asarray(exclude, dtype=bool)[np.minimum(ind, ny * nx - 1)] == 0
    if npix > 1:
        w = np.exp(-D ** 2 / (2 * (0.5 * dmax) ** 2)) * valid
        s = w.sum(axis=1, keepdims=True)
        w = np.divide(w, s, out=np.zeros_like(w), where=s > 0)
    else:
        w = np.ones_like(D)
    idx = np.where(valid, ind, -1).astype(np.int64)
    w = np.where(valid, w, 0.0)
    return idx, w


def interp_rows_gpu(x_km, y_km, ny, nx, dx, dy, npix=4, device="cuda", exclude=None):
    """interp_rows on the GPU (vd_obs_knn, or vd_obs_knn_excl with an
    ``exclude`` table); returns host arrays (idx with -1 for dropped
    neighbours, w), shapes [n, npix]."""
    x = torch.as_tensor(np.ascontiguousarray(x_km, dtype=np.float64), device=device)
    y = torch.as_tensor(np.ascontiguousarray(y_km, dtype=np.float64), device=device)
    n = x.numel()
    idx = torch.empty((max(n, 1), 4), dtype=torch.int64, device=device)
    w = torch.empty((max(n, 1), 4), dtype=torch.float64, device=device)
    if exclude is None:
        _lib.call("vd_obs_knn", n, _p(x), _p(y), ny, nx, dx / 1e3, dy / 1e3, npix, dmax_km(dx, dy, npix), _p(idx),
                  _p(w), _stream())
    else:
        ex = np.ascontiguousarray(exclude, dtype=np.uint8).reshape(-1)
        if ex.size != ny * nx:
            raise ValueError("exclude holds one byte per grid point")
        ex = torch.as_tensor(ex, device=device)
        _lib.call("vd_obs_knn_excl", n, _p(x), _p(y), ny, nx, dx / 1e3, dy / 1e3, npix, dmax_km(dx, dy, npix),
                  _p(ex), _p(idx), _p(w), _stream())
    return idx[:n, :npix].cpu().numpy(), w[:n, :npix].cpu().numpy()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class AlongTrackObs:
    """Observations of ``B`` windows on one (ny, nx) grid.

    ``windows[b]`` is a dict with arrays ``x_km``, ``y_km`` (planar position),
    ``step`` (model step index at which the point is observed), ``yobs`` and
    ``err`` (observation error, the reference's ``errobs``). ``exclude`` (an
    :func:`l3_exclusion` table) builds the scipy operator ``Obsop_interp_l3``
    instead (obsop.py:161-373): same misfit, same gradient of the cost, and
    neighbours on excluded grid points dropped."""

    def __init__(self, windows, ny, nx, dx, dy, dtype=torch.float32, device="cuda", npix=4, build="gpu",
                 exclude=None, operator=None):
        """``operator`` (optional): one ``(idx, w)`` pair per window, arrays
        [n, npix] of grid indices (-1 for no neighbour) and weights, for
        operators built elsewhere (e.g. the reference's 3-D Cartesian
        distances on a lon/lat grid); ``x_km`` / ``y_km`` are then unused."""
        if npix > 4:
            raise ValueError("at most 4 neighbours per observation")
        if build not in ("gpu", "host"):
            raise ValueError("build is 'gpu' or 'host'")
        if operator is not None and len(operator) != len(windows):
            raise ValueError("one (idx, w) operator per window")
        rows = interp_rows_gpu if build == "gpu" else interp_rows
        self.B = len(windows)
        self.ny, self.nx = ny, nx
        self.dtype = dtype
        self.vd_dtype = _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32
        self.device = torch.device(device)
        fields, steps, idxs, ws, ys, errs = [], [], [], [], [], []
        for b, win in enumerate(windows):
            if operator is not None:
                idx = np.asarray(operator[b][0], dtype=np.int64).reshape(len(win["step"]), -1)
                w = np.asarray(operator[b][1], dtype=np.float64).reshape(idx.shape)
                if idx.shape[1] != npix:
                    raise ValueError(f"operator rows of window {b} have {idx.shape[1]} entries, npix is {npix}")
                x = idx[:, 0]
            else:
                x = np.asarray(win["x_km"], dtype=np.float64)
                idx, w = rows(x, np.asarray(win["y_km"], dtype=np.float64), ny, nx, dx, dy, npix, exclude=exclude)
            pad = 4 - npix
            if pad:
                idx = np.pad(idx, ((0, 0), (0, pad)), constant_values=-1)
                w = np.pad(w, ((0, 0), (0, pad)))
            fields.append(np.full(x.size, b, dtype=np.int64))
            steps.append(np.asarray(win["step"], dtype=np.int64))
            idxs.append(idx)
            ws.append(w)
            ys.append(np.asarray(win["yobs"], dtype=np.float64))
            errs.append(np.asarray(win["err"], dtype=np.float64))
        field = np.concatenate(fields)
        step = np.concatenate(steps)
        idx = np.concatenate(idxs)
        w = np.concatenate(ws)
        y = np.concatenate(ys)
        err = np.concatenate(errs)
        order = np.lexsort((field, step))           # time-major, then window
        field, step, idx, w, y, err = field[order], step[order], idx[order], w[order], y[order], err[order]
        self.nobs = field.size
        self.obs_window = field
        self.obs_step = step
        with np.errstate(divide="ignore", invalid="ignore"):
            inverr = 1.0 / err
        inverr = np.where(np.isnan(inverr), 0.0, inverr)

        # per-step ranges
        self.steps = np.unique(step)
        starts = np.searchsorted(step, self.steps, side="left")
        ends = np.searchsorted(step, self.steps, side="right")
        self.step_range = {int(s): (int(a), int(e)) for s, a, e in zip(self.steps, starts, ends)}

        # CSR transpose per step: rows = unique (window, grid index)
        pt_field, pt_index, rowptr, ent_obs, ent_w = [], [], [0], [], []
        self.step_pts = {}
        for s in self.steps:
            a, e = self.step_range[int(s)]
            o = np.repeat(np.arange(a, e), 4)
            g = idx[a:e].ravel()
            ww = w[a:e].ravel()
            fb = np.repeat(field[a:e], 4)
            keep = g >= 0
            o, g, ww, fb = o[keep], g[keep], ww[keep], fb[keep]
            key = fb * (ny * nx) + g
            srt = np.argsort(key, kind="stable")
            key, o, ww = key[srt], o[srt], ww[srt]
            uk, first = np.unique(key, return_index=True)
            p0 = len(pt_field)
            pt_field.extend((uk // (ny * nx)).tolist())
            pt_index.extend((uk % (ny * nx)).tolist())
            bounds = list(first[1:]) + [key.size]
            base = len(ent_obs)
            rowptr.extend((base + np.asarray(bounds)).tolist())
            ent_obs.extend(o.tolist())
            ent_w.extend(ww.tolist())
            self.step_pts[int(s)] = (p0, len(pt_field))

        # per-window segments in time-major storage for Jo
        perm = np.argsort(field, kind="stable")
        win_off = np.searchsorted(field[perm], np.arange(self.B + 1), side="left")

        dev = self.device
        i32 = lambda a: torch.as_tensor(np.asarray(a, dtype=np.int32), device=dev)
        flt = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev).to(dtype)
        self.d_field = i32(field)
        self.d_idx4 = i32(idx.reshape(-1))
        self.d_w4 = flt(w.reshape(-1))
        self.d_y = flt(y)
        self.d_inverr = flt(inverr)
        self.d_pt_field = i32(pt_field)
        self.d_pt_index = i32(pt_index)
        self.d_rowptr = i32(rowptr)
        self.d_ent_obs = i32(ent_obs)
        self.d_ent_w = flt(ent_w)
        self.d_perm = i32(perm)
        self.d_win_off = i32(win_off)
        self.misfit = torch.zeros(max(self.nobs, 1), dtype=dtype, device=dev)
        self.host = dict(field=field, step=step, idx=idx, w=w, y=y, inverr=inverr)

    # -------- kernels --------
    def apply_misfit(self, s, fields):
        """misfit of the observations of step ``s`` from ``fields`` [B, ny, nx]."""
        a, e = self.step_range[int(s)]
        if e <= a:
            return
        es = self.d_w4.element_size()
        _lib.call("vd_obs_misfit", self.vd_dtype, e - a, _p(fields), ctypes.c_longlong(self.ny * self.nx),
                  ctypes.c_void_p(self.d_field.data_ptr() + 4 * a),
                  ctypes.c_void_p(self.d_idx4.data_ptr() + 16 * a),
                  ctypes.c_void_p(self.d_w4.data_ptr() + 4 * es * a),
                  ctypes.c_void_p(self.d_y.data_ptr() + es * a),
                  ctypes.c_void_p(self.d_inverr.data_ptr() + es * a),
                  ctypes.c_void_p(self.misfit.data_ptr() + es * a), _stream())

    def apply_adjoint(self, s, ad_fields, cot=None):
        """ad_fields[b] += H_s^T (inverr * cot) for the observations of step s
        (cot defaults to the stored misfit, as the reference's adj does)."""
        p0, p1 = self.step_pts.get(int(s), (0, 0))
        if p1 <= p0:
            return
        cot = self.misfit if cot is None else cot
        _lib.call("vd_obs_adjoint", self.vd_dtype, p1 - p0, _p(ad_fields), ctypes.c_longlong(self.ny * self.nx),
                  ctypes.c_void_p(self.d_pt_field.data_ptr() + 4 * p0),
                  ctypes.c_void_p(self.d_pt_index.data_ptr() + 4 * p0),
                  ctypes.c_void_p(self.d_rowptr.data_ptr() + 4 * p0),
                  _p(self.d_ent_obs), _p(self.d_ent_w), _p(self.d_inverr), _p(cot), _stream())

    def sumsq_per_window(self, out, scale=1.0):
        """out[b] = scale * sum of misfit^2 over window b (FP64)."""
        _lib.call("vd_sumsq_gather_f64", self.vd_dtype, self.B, _p(self.d_win_off), _p(self.d_perm),
                  _p(self.misfit), float(scale), _p(out), _stream())
