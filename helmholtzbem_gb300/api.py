"""Python mirror of the reference's API for the assembly-and-resonance path.

Names, argument meaning and error behaviour follow the reference classes
(include/galerkin_builder.hpp, include/gen_sol_op.hpp, include/singular_values.hpp,
include/find_roots.hpp); every call goes through the C ABI of libhbem.so.
"""
import ctypes
import os

import numpy as np

from . import _capi as C
from ._capi import check, dptr, iptr

LayerType_DOUBLE = C.LAYER_DOUBLE
LayerType_SINGLE = C.LAYER_SINGLE
LayerType_HYPERSINGULAR = C.LAYER_HYPERSINGULAR
LayerType_ALL = C.LAYER_ALL


class BuilderData:
    """BuilderData(mesh, test_space, trial_space, order); mesh = (kinds, params)."""

    def __init__(self, mesh, test_space=C.SPACE_P1, trial_space=C.SPACE_P1, order=11):
        kinds, params = mesh
        self.kinds = np.ascontiguousarray(kinds, np.int32)
        self.params = np.ascontiguousarray(params, np.float64).reshape(-1, 5)
        self.order = int(order)
        h = ctypes.c_void_p()
        check(C.lib().hbem_builder_create(int(self.kinds.size), iptr(self.kinds), dptr(self.params), self.order,
                                          int(test_space), int(trial_space), ctypes.byref(h)))
        self._h = h
        n, dt, dr, o, ln = (ctypes.c_int() for _ in range(5))
        check(C.lib().hbem_builder_info(self._h, ctypes.byref(n), ctypes.byref(dt), ctypes.byref(dr), ctypes.byref(o),
                                        ctypes.byref(ln)))
        self.npanels, self.dim_test, self.dim_trial = n.value, dt.value, dr.value
        self.panels_are_lines = bool(ln.value)

    def getNumPanels(self):
        return self.npanels

    def getTestSpaceDimension(self):
        return self.dim_test

    def getTrialSpaceDimension(self):
        return self.dim_trial

    def getPanelsAreLines(self):
        return self.panels_are_lines

    def is_adjacent(self, i, j):
        a, s = ctypes.c_int(), ctypes.c_int()
        check(C.lib().hbem_builder_is_adjacent(self._h, i, j, ctypes.byref(a), ctypes.byref(s)))
        return bool(a.value), bool(s.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and C._lib is not None:
            C._lib.hbem_builder_destroy(h)
            self._h = None


class GalerkinBuilder:
    """GalerkinBuilder(data): assembleDense + layer getters (complex128, N x N)."""

    def __init__(self, data: BuilderData):
        self.data = data

    def assembleDense(self, k, c, layers=LayerType_ALL, d=0, row=0, col=0, rows=0, cols=0):
        k = complex(k)
        n = self.data.npanels
        self._shape = (rows or n, cols or n)
        check(C.lib().hbem_assemble_dense_sub(self.data._h, k.real, k.imag, float(c), int(layers), int(d), int(row),
                                              int(col), int(rows), int(cols)))

    def _get(self, layer, d):
        n = self.data.npanels
        out = np.zeros(getattr(self, "_shape", (n, n)), np.complex128, order="F")
        check(C.lib().hbem_get_layer(self.data._h, layer, int(d), out.ctypes.data_as(C._dp)))
        return out

    def getDoubleLayer(self, d=0):
        return self._get(C.LAYER_DOUBLE, d)

    def getHypersingular(self, d=0):
        return self._get(C.LAYER_HYPERSINGULAR, d)

    def getSingleLayer(self, d=0):
        return self._get(C.LAYER_SINGLE, d)


class SolutionsOperator:
    """SolutionsOperator(builder_data, proj=True)."""

    def __init__(self, data: BuilderData, proj=True):
        self.data = data
        h = ctypes.c_void_p()
        check(C.lib().hbem_solop_create(data._h, 1 if proj else 0, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and C._lib is not None:
            C._lib.hbem_solop_destroy(h)
            self._h = None

    def mass_matrix(self):
        n = self.data.npanels
        M = np.zeros((n, n), order="F")
        check(C.lib().hbem_mass_matrix(self._h, M.ctypes.data_as(C._dp)))
        return M

    def _gen(self, k, c_o, c_i, d):
        k = complex(k)
        n = 2 * self.data.npanels
        buf = np.zeros((d + 1, n, n), np.complex128)   # each matrix column-major => transpose views
        check(C.lib().hbem_gen_sol_op(self._h, k.real, k.imag, float(c_o), float(c_i), int(d),
                                      buf.ctypes.data_as(C._dp)))
        return [buf[t].T for t in range(d + 1)]

    def gen_sol_op(self, k, c_o, c_i):
        return self._gen(k, c_o, c_i, 0)[0]

    def gen_sol_op_1st_der(self, k, c_o, c_i):
        return tuple(self._gen(k, c_o, c_i, 1))

    def gen_sol_op_2nd_der(self, k, c_o, c_i):
        return tuple(self._gen(k, c_o, c_i, 2))

    def sweep_sigma(self, ks, c_o, c_i, d=2):
        ks = np.ascontiguousarray(ks, np.float64)
        out = np.zeros((ks.size, 3))
        check(C.lib().hbem_sweep_sigma(self._h, dptr(ks), int(ks.size), float(c_o), float(c_i), int(d), dptr(out)))
        return out

    def sigma_rsvd_sweep(self, ks, c_o, c_i, sketch=2, q=2, precision=0, seed=0):
        """randomized_svd::sv along ks on a seeded sketch of width `sketch`."""
        ks = np.ascontiguousarray(ks, np.float64)
        out = np.zeros(ks.size)
        check(C.lib().hbem_sigma_rsvd_sweep(self._h, dptr(ks), int(ks.size), float(c_o), float(c_i), int(sketch),
                                            int(q), int(precision), int(seed), dptr(out)))
        return out

    def find_resonances_adaptive(self, k_min, k_max, c_o, c_i, batch_size=16, limit=10, sample_tol=None, tol=1e-6,
                                 seed=0, sketch=2, q=2, max_roots=4096):
        """examples/find_resonances.cpp's search: opt_subdiv sampling, rational
        interpolation, Brent refinement.  Returns (roots, n_samples, n_evals)."""
        if sample_tol is None:
            sample_tol = 1e-4 * (k_max - k_min)
        roots = np.zeros(max_roots)
        nr, ns, ne = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(C.lib().hbem_find_resonances_adaptive(self._h, float(k_min), float(k_max), float(c_o), float(c_i),
                                                    int(batch_size), int(limit), float(sample_tol), float(tol),
                                                    int(seed), int(sketch), int(q), dptr(roots), int(max_roots),
                                                    ctypes.byref(nr), ctypes.byref(ns), ctypes.byref(ne)))
        return roots[:min(nr.value, max_roots)].copy(), ns.value, ne.value

    def refine_brackets(self, a, b, c_o, c_i, tol=1e-8, max_shift=3, max_roots=4096):
        """Local minima of sigma_min from candidate brackets [a_i, b_i]: (roots, n_evals)."""
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        out = np.zeros(max_roots)
        nr, ne = ctypes.c_int(), ctypes.c_int()
        check(C.lib().hbem_refine_brackets(self._h, dptr(a), dptr(b), int(a.size), float(c_o), float(c_i), float(tol),
                                           int(max_shift), dptr(out), max_roots, ctypes.byref(nr), ctypes.byref(ne)))
        return out[:min(nr.value, max_roots)].copy(), ne.value

    def find_resonances_plain_verified(self, k_min, k_max, npoints, c_o, c_i, tol=1e-8, max_roots=4096):
        """The plain search with every root checked: (roots, grid, evaluations, check),
        check[i] = sigma' at roots[i] - tol and roots[i] + tol; a root is verified when
        check[i, 0] <= 0 <= check[i, 1]."""
        roots = np.zeros(max_roots)
        grid = np.zeros((npoints, 3))
        chk = np.zeros((max_roots, 2))
        nr, ne = ctypes.c_int(), ctypes.c_int()
        check(C.lib().hbem_find_resonances_plain_verified(self._h, float(k_min), float(k_max), int(npoints),
                                                          float(c_o), float(c_i), float(tol), dptr(roots), max_roots,
                                                          ctypes.byref(nr), dptr(grid), ctypes.byref(ne), dptr(chk)))
        m = min(nr.value, max_roots)
        return roots[:m].copy(), grid, ne.value, chk[:m].copy()

    def find_resonances_plain(self, k_min, k_max, npoints, c_o, c_i, tol=1e-8, max_roots=4096):
        roots = np.zeros(max_roots)
        grid = np.zeros((npoints, 3))
        nr, ne = ctypes.c_int(), ctypes.c_int()
        check(C.lib().hbem_find_resonances_plain(self._h, float(k_min), float(k_max), int(npoints), float(c_o),
                                                 float(c_i), float(tol), dptr(roots), max_roots, ctypes.byref(nr),
                                                 dptr(grid), ctypes.byref(ne)))
        return roots[:min(nr.value, max_roots)].copy(), grid, ne.value


def sv_dense(Ts, d=0, all_values=False):
    """direct::sv / sv_1st_der / sv_2nd_der for a batch: Ts is a list (one per matrix)
    of [T] / [T, T'] / [T, T', T''].  Returns (nmat, 3) [sigma_min, sigma', sigma'']."""
    nmat = len(Ts)
    n = Ts[0][0].shape[0]
    buf = np.zeros((nmat, d + 1, n, n), np.complex128)
    for m, mats in enumerate(Ts):
        for t in range(d + 1):
            buf[m, t] = np.asarray(mats[t]).T      # column-major
    out = np.zeros((nmat, 3))
    sig = np.zeros((nmat, n)) if all_values else None
    check(C.lib().hbem_sv_dense_batch(n, nmat, int(d), buf.ctypes.data_as(C._dp), dptr(out),
                                      dptr(sig) if all_values else None))
    return (out, sig) if all_values else out


def rtsafe(f, f_both, x1, x2, tol):
    """rtsafe(f, f_both, x1, x2, tol) -> (root, root_found, num_iter); f_both(x) -> (f, f')."""
    cb = C.FN(lambda x, u: float(f(x)))

    def _both(x, pf, pdf, u):
        a, b = f_both(x)
        pf[0] = float(a)
        pdf[0] = float(b)

    cbb = C.FN_BOTH(_both)
    rf, ni = ctypes.c_int(), ctypes.c_uint()
    r = C.lib().hbem_rtsafe(cb, cbb, None, float(x1), float(x2), float(tol), ctypes.byref(rf), ctypes.byref(ni))
    return r, bool(rf.value), ni.value


def zbrent(f, x1, x2, tol):
    cb = C.FN(lambda x, u: float(f(x)))
    rf, ni = ctypes.c_int(), ctypes.c_uint()
    r = C.lib().hbem_zbrent(cb, None, float(x1), float(x2), float(tol), ctypes.byref(rf), ctypes.byref(ni))
    return r, bool(rf.value), ni.value


def brent_min(f, a, b, tol):
    cb = C.FN(lambda x, u: float(f(x)))
    return C.lib().hbem_brent_min(cb, None, float(a), float(b), float(tol))


class BrentMinimizer:
    """BrentMinimizer(a, b, tol).local_min_rc(status, value) with reverse
    communication (include/find_roots.hpp:181-233): returns (arg, status)."""

    def __init__(self, a, b, tol):
        if not a < b:
            raise RuntimeError("a < b is required for Brent algorithm!")
        h = ctypes.c_void_p()
        check(C.lib().hbem_brent_rc_create(float(a), float(b), float(tol), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and C._lib is not None:
            C._lib.hbem_brent_rc_destroy(self._h)
            self._h = None

    def local_min_rc(self, status, value=0.0):
        st = ctypes.c_int(int(status))
        arg = C.lib().hbem_brent_rc_step(self._h, ctypes.byref(st), float(value))
        return arg, st.value


def brent_guess(a, b, guess, fguess, f, tol):
    cb = C.FN(lambda x, u: float(f(x)))
    ic = ctypes.c_uint()
    r = C.lib().hbem_brent_guess(cb, None, float(a), float(b), float(guess), float(fguess), float(tol), ctypes.byref(ic))
    return r, ic.value


def brent_gsl_with_values(a, fa, b, fb, guess, fguess, f, tol):
    cb = C.FN(lambda x, u: float(f(x)))
    ic = ctypes.c_uint()
    r = C.lib().hbem_brent_gsl_with_values(cb, None, float(a), float(fa), float(b), float(fb), float(guess),
                                           float(fguess), float(tol), ctypes.byref(ic))
    return r, ic.value


def hankel01(z):
    """H0^(1), H1^(1) on the device; real path for a real array, complex path otherwise."""
    z = np.asarray(z)
    cplx_arg = not np.isrealobj(z)
    src = np.ascontiguousarray(z.ravel(), np.complex128 if cplx_arg else np.float64)
    h0 = np.zeros(src.size, np.complex128)
    h1 = np.zeros(src.size, np.complex128)
    check(C.lib().hbem_hankel01(int(src.size), src.ctypes.data_as(C._dp), 1 if cplx_arg else 0,
                                h0.ctypes.data_as(C._dp), h1.ctypes.data_as(C._dp)))
    return h0.reshape(z.shape), h1.reshape(z.shape)


def randGaussian(nr, nc, seed=0):
    """randomized_svd::randGaussian: (U[0,1] + i U[0,1])/sqrt2, seeded."""
    R = np.zeros((nc, nr), np.complex128)        # column-major nr x nc
    check(C.lib().hbem_rand_sketch(int(nr), int(nc), int(seed), R.ctypes.data_as(C._dp)))
    return R.T


def rsvd_sv(Ts, R, q=0, d=0):
    """randomized_svd::sv (d = 0) / sv_der (d = 1) / sv_der2 (d = 2) for a batch: Ts
    is a list of [T], [T, T'] or [T, T', T''].  Returns (nmat, d + 1): sigma estimate,
    sigma', sigma''."""
    nmat = len(Ts)
    n = Ts[0][0].shape[0]
    R = np.asarray(R, np.complex128)
    s = R.shape[1]
    buf = np.zeros((nmat, d + 1, n, n), np.complex128)
    for m, mats in enumerate(Ts):
        for t in range(d + 1):
            buf[m, t] = np.asarray(mats[t]).T
    Rc = np.ascontiguousarray(R.T)                 # column-major n x s
    out = np.zeros((nmat, d + 1))
    check(C.lib().hbem_rsvd_sv_batch(n, nmat, int(d), buf.ctypes.data_as(C._dp), Rc.ctypes.data_as(C._dp), int(s),
                                     int(q), dptr(out)))
    return out

def arnoldi_sv(Ts, count=1, acc=0.0, d=0, return_status=False):
    """arnoldi::sv (d = 0) / sv_1st_der (d = 1) / sv_2nd_der (d = 2) for a batch
    (include/singular_values_arnoldi.hpp:29-66): Ts is a list of [T], [T, T'] or
    [T, T', T''].  Returns (nmat, count, d + 1): the count smallest singular values
    in ascending order with their derivatives.  A matrix whose iteration reaches the
    cap keeps its last iterate and raises HbemError (status 4) unless return_status
    is set, in which case (values, status, ...) is returned with per-matrix status
    0 converged / 5 singular / 6 iteration cap."""
    nmat = len(Ts)
    n = Ts[0][0].shape[0]
    buf = np.zeros((nmat, d + 1, n, n), np.complex128)
    for m, mats in enumerate(Ts):
        for t in range(d + 1):
            buf[m, t] = np.asarray(mats[t]).T
    out = np.zeros((nmat, count, d + 1))
    status = np.zeros(nmat, np.int32)
    rc = C.lib().hbem_arnoldi_sv_batch(n, nmat, int(d), int(count), float(acc), buf.ctypes.data_as(C._dp),
                                       dptr(out), iptr(status))
    if return_status:
        if rc not in (0, 4, 5):
            check(rc)
        return out, status
    check(rc)
    return out

# ---------------------------------------------------------------- incoming waves, transmission problem

WAVE_TYPES = {"Plane": 0, "CircularJ": 1, "CircularY": 2, "FourierHankel1": 3, "FourierHankel2": 4, "Herglotz": 5}


def wave(kind, amplitude=1.0, x0=(0.0, 0.0), angle=0.0, eps=0.0, order=0):
    """One incoming-wave record (incoming::wavespec_t): kind is a WAVE_TYPES name."""
    return np.array([WAVE_TYPES[kind], amplitude, x0[0], x0[1], angle, eps, order], np.float64)


def _waves(waves):
    w = np.ascontiguousarray(np.asarray(waves, np.float64).reshape(-1, 7))
    return w, w.shape[0]


def incoming_load(fname):
    """incoming::load: the wave records of a file; raises ValueError where the
    reference returns false."""
    n = ctypes.c_int()
    if C.lib().hbem_incoming_load(os.fsencode(fname), None, 0, ctypes.byref(n)) != 0:
        raise ValueError("failed to read incoming wave from file " + str(fname))
    out = np.zeros((n.value, 7))
    check(C.lib().hbem_incoming_load(os.fsencode(fname), dptr(out), n.value, ctypes.byref(n)))
    return out


def incoming_eval(waves, k, xy):
    """incoming::compute and compute_del at the points xy (m x 2): (u (m), grad (m x 2))."""
    w, nw = _waves(waves)
    k = complex(k)
    xy = np.ascontiguousarray(np.asarray(xy, np.float64).reshape(-1, 2))
    m = xy.shape[0]
    u = np.zeros(m, np.complex128)
    du = np.zeros((m, 2), np.complex128)
    check(C.lib().hbem_incoming_eval(dptr(w), nw, k.real, k.imag, dptr(xy), m, u.ctypes.data_as(C._dp),
                                     du.ctypes.data_as(C._dp)))
    return u, du


def tp_solve(solop, waves, k, c_o, c_i):
    """tp::direct_second_kind::solve: the 2N traces (Dirichlet, Neumann) of the
    transmission problem for the incoming wave; solop must be unprojected."""
    w, nw = _waves(waves)
    k = complex(k)
    out = np.zeros(2 * solop.data.npanels, np.complex128)
    check(C.lib().hbem_tp_solve(solop._h, dptr(w), nw, k.real, k.imag, float(c_o), float(c_i),
                                out.ctypes.data_as(C._dp)))
    return out


def tp_field_grid(solop, waves, k, c_o, c_i, order_green, lower_left, upper_right, nx, ny, total_field=False,
                  traces=None):
    """tp::direct_second_kind::solve_in_rectangle: (S, grid_X, grid_Y), each nx x ny,
    S[i, j] the field at (grid_X[i, j], grid_Y[i, j])."""
    w, nw = _waves(waves)
    k = complex(k)
    S = np.zeros((ny, nx), np.complex128)
    gx = np.zeros((ny, nx))
    gy = np.zeros((ny, nx))
    tr = None
    if traces is not None:
        tr = np.ascontiguousarray(np.asarray(traces, np.complex128))
    check(C.lib().hbem_tp_field_grid(solop._h, dptr(w), nw, k.real, k.imag, float(c_o), float(c_i), int(order_green),
                                     float(lower_left[0]), float(lower_left[1]), float(upper_right[0]),
                                     float(upper_right[1]), int(nx), int(ny), 1 if total_field else 0,
                                     tr.ctypes.data_as(C._dp) if tr is not None else None,
                                     S.ctypes.data_as(C._dp), dptr(gx), dptr(gy)))
    return S.T.copy(), gx.T.copy(), gy.T.copy()


# ---------------------------------------------------------------- many scatterers at once

def _ops(ops):
    return (ctypes.c_void_p * len(ops))(*[o._h.value for o in ops])


def sweep_sigma_multi(ops, ks, c_o, c_i, d=0):
    """sigma (and derivatives up to d) of operator i at the wavenumbers ks[i] with inner
    index c_i[i], all scatterers in flight together: list of (len(ks[i]), 3) arrays."""
    counts = np.array([len(k) for k in ks], np.int32)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(k, np.float64) for k in ks]))
    ci = np.ascontiguousarray(c_i, np.float64)
    out = np.zeros((flat.size, 3))
    check(C.lib().hbem_sweep_sigma_multi(_ops(ops), len(ops), iptr(counts), dptr(flat), dptr(ci), float(c_o), int(d),
                                         dptr(out)))
    return np.split(out, np.cumsum(counts)[:-1])


def gen_sol_op_multi_device(ops, ks, c_o, c_i, d=0, out=None):
    """T(k) and its first d derivatives of operator i at the wavenumbers ks[i] (inner
    index c_i[i]) on the device, every scatterer's panel-pair quadrature in the same
    launches: list of torch tensors [len(ks[i]), d + 1, 2N_i, 2N_i] (complex128,
    each matrix column-major, i.e. the transposes of the row-major views)."""
    import torch
    counts = np.array([len(k) for k in ks], np.int32)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(k, np.float64) for k in ks]))
    ci = np.ascontiguousarray(c_i, np.float64)
    if out is None:
        out = [torch.empty((len(k), d + 1, 2 * o.data.npanels, 2 * o.data.npanels), dtype=torch.complex128,
                           device="cuda") for o, k in zip(ops, ks)]
    ptrs = (ctypes.c_void_p * len(ops))(*[t.data_ptr() for t in out])
    check(C.lib().hbem_gen_sol_op_multi_device(_ops(ops), len(ops), iptr(counts), dptr(flat), dptr(ci), float(c_o),
                                               int(d), ptrs))
    return out


def _split_roots(roots, counts):
    return np.split(roots[:int(np.sum(counts))].copy(), np.cumsum(counts)[:-1])


def find_resonances_plain_multi(ops, k_min, k_max, npoints, c_o, c_i, tol=1e-8, max_roots=65536):
    """The plain search on window [k_min[i], k_max[i]] of operator i, all in lock step:
    (list of root arrays, sigma evaluations)."""
    n = len(ops)
    roots = np.zeros(max_roots)
    counts = np.zeros(n, np.int32)
    ne = ctypes.c_int()
    check(C.lib().hbem_find_resonances_plain_multi(_ops(ops), n, dptr(np.ascontiguousarray(k_min, np.float64)),
                                                   dptr(np.ascontiguousarray(k_max, np.float64)), int(npoints),
                                                   float(c_o), dptr(np.ascontiguousarray(c_i, np.float64)),
                                                   float(tol), dptr(roots), max_roots, iptr(counts), ctypes.byref(ne)))
    return _split_roots(roots, counts), ne.value


def refine_brackets_multi(ops, a, b, c_o, c_i, tol=1e-8, max_shift=3, max_roots=65536):
    """hbem_refine_brackets for every operator in lock step: brackets a[i], b[i] of
    operator i: (list of root arrays, sigma evaluations)."""
    n = len(ops)
    counts = np.array([len(x) for x in a], np.int32)
    af = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in a]) if n else np.zeros(0))
    bf = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in b]) if n else np.zeros(0))
    roots = np.zeros(max_roots)
    rc = np.zeros(n, np.int32)
    ne = ctypes.c_int()
    check(C.lib().hbem_refine_brackets_multi(_ops(ops), n, iptr(counts), dptr(af), dptr(bf), float(c_o),
                                             dptr(np.ascontiguousarray(c_i, np.float64)), float(tol), int(max_shift),
                                             dptr(roots), max_roots, iptr(rc), ctypes.byref(ne)))
    return _split_roots(roots, rc), ne.value


# ---------------------------------------------------------------- proposal network

class MLP:
    """The learned proposal's network (BF16 products, FP32 accumulation and master
    weights, Adam) on the GPU: n_in -> width (GELU) x depth -> n_out."""

    def __init__(self, n_in, width, depth, n_out, seed=0):
        self.dims = [n_in] + [width] * depth + [n_out]
        h = ctypes.c_void_p()
        check(C.lib().hbem_mlp_create(int(n_in), int(width), int(depth), int(n_out), int(seed), ctypes.byref(h)))
        self._h = h
        c = ctypes.c_longlong()
        check(C.lib().hbem_mlp_num_params(self._h, ctypes.byref(c)))
        self.num_params = c.value

    def __del__(self):
        if getattr(self, "_h", None) and C._lib is not None:
            C._lib.hbem_mlp_destroy(self._h)
            self._h = None

    @staticmethod
    def _f(a):
        return np.ascontiguousarray(np.asarray(a, np.float32))

    def get_params(self):
        p = np.zeros(self.num_params, np.float32)
        check(C.lib().hbem_mlp_get_params(self._h, p.ctypes.data_as(C._fp)))
        return p

    def set_params(self, p):
        p = self._f(p)
        check(C.lib().hbem_mlp_set_params(self._h, p.ctypes.data_as(C._fp)))

    def forward(self, X):
        X = self._f(X)
        Y = np.zeros((X.shape[0], self.dims[-1]), np.float32)
        check(C.lib().hbem_mlp_forward(self._h, X.ctypes.data_as(C._fp), X.shape[0], Y.ctypes.data_as(C._fp)))
        return Y

    def gradients(self, X, T):
        X, T = self._f(X), self._f(T)
        g = np.zeros(self.num_params, np.float32)
        loss = ctypes.c_float()
        check(C.lib().hbem_mlp_gradients(self._h, X.ctypes.data_as(C._fp), T.ctypes.data_as(C._fp), X.shape[0],
                                         ctypes.byref(loss), g.ctypes.data_as(C._fp)))
        return loss.value, g

    def train_step(self, X, T, lr):
        X, T = self._f(X), self._f(T)
        loss = ctypes.c_float()
        check(C.lib().hbem_mlp_train_step(self._h, X.ctypes.data_as(C._fp), T.ctypes.data_as(C._fp), X.shape[0],
                                          float(lr), ctypes.byref(loss)))
        return loss.value


def opt_subdiv(f, x_min, x_max, batch_size, limit, tol, seed=0, max_points=100000):
    """opt_subdiv for a batched Python function f(xs) -> ys: returns (x, y, minima)."""
    def _f(xp, n, yp, user):
        xs = np.ctypeslib.as_array(xp, shape=(n,)).copy()
        ys = np.asarray(f(xs), np.float64)
        for i in range(n):
            yp[i] = float(ys[i])

    cb = C.FN_BATCH(_f)
    x = np.zeros(max_points)
    y = np.zeros(max_points)
    mins = np.zeros(max_points, np.int32)
    npnt, nmin = ctypes.c_int(), ctypes.c_int()
    check(C.lib().hbem_opt_subdiv(cb, None, float(x_min), float(x_max), int(batch_size), int(limit), float(tol),
                                  int(seed), dptr(x), dptr(y), max_points, ctypes.byref(npnt), iptr(mins), max_points,
                                  ctypes.byref(nmin)))
    n = min(npnt.value, max_points)
    return x[:n].copy(), y[:n].copy(), mins[:min(nmin.value, max_points)].copy()
