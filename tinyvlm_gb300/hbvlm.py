"""Harmonic-balance VLM: the ``libhbvlm`` (2-DOF) and ``libhbvlm3`` (3-DOF
wing + flap) Python modules of the reference, over the gbvlm C ABI.

Mirrors lib/libhbvlm.cpp and lib/libhbvlm3.cpp: ``HBVLM(backend, mesh(es))``,
``.init(harmonics, scaling)``, ``.run(omega, [U,] dyn_f, forces_t)`` with
``forces_t`` filled in place.  The kinematics (heave / pitch / flap Fourier
series) are evaluated here with dual numbers; the fixed-point map, Anderson
acceleration and loads run in the library (double precision).  The
circulation coefficients persist between ``run`` calls and seed the next
fixed point, as in the reference.
"""
import ctypes
import math

import numpy as np

from . import _lib
from ._lib import P, PP, call, dims_array
from .kinematics import Assembly, KinematicsTree, cos, rotation_matrix, sin, translation_matrix
from .vlm import read_plot3d

PI_F = float(np.float32(3.141593))
TWO_PI_F = float(np.float32(2.0) * np.float32(3.141593))  # 2.0f * PI_f as the reference forms it


def dft_matrices(N, omega, period):
    """Scaled orthonormal DFT and its time derivative (libhbvlm3.cpp:322-347), column-major (N x N)."""
    s0 = 1.0 / math.sqrt(N)
    s2 = math.sqrt(2.0 / N)
    D = np.zeros((N, N))
    DD = np.zeros((N, N))
    D[:, 0] = s0
    for j in range(1, N, 2):
        k = (j + 1) / 2.0
        for i in range(N):
            tn = (i / N) * period
            D[i, j] = math.cos(omega * tn * k) * s2
            D[i, j + 1] = math.sin(omega * tn * k) * s2
            DD[i, j] = -omega * k * math.sin(omega * tn * k) * s2
            DD[i, j + 1] = omega * k * math.cos(omega * tn * k) * s2
    return np.asfortranarray(D), np.asfortranarray(DD)


def fourier(row, H, omega, t):
    """r(row, 0) + sum_h cos(w t k) r(row, 2h+1) + sin(w t k) r(row, 2h+2) on a dual t."""
    z = row[0] + 0.0 * t
    for h in range(H):
        k = float(h + 1)
        z = z + cos(omega * t * k) * row[2 * h + 1] + sin(omega * t * k) * row[2 * h + 2]
    return z


def last_panel_chord(v):
    d = v[:3, -1, 0].astype(np.float64) - v[:3, -2, 0].astype(np.float64)
    return math.sqrt(float(d @ d))


class HBEngine:
    """gbvlm_hbvlm_* handle for a set of surfaces (exactly one lifting)."""

    def __init__(self, verts, lifting):
        self.verts = [np.ascontiguousarray(v, np.float64) for v in verts]
        self.lifting = list(lifting)
        self.n = sum((v.shape[1] - 1) * (v.shape[2] - 1) for v in self.verts)
        d = dims_array([(v.shape[2] - 1, v.shape[1] - 1, 0) for v in self.verts])
        arr = (ctypes.c_void_p * len(self.verts))(*[v.ctypes.data for v in self.verts])
        lf = (ctypes.c_int32 * len(self.verts))(*[1 if x else 0 for x in self.lifting])
        h = ctypes.c_void_p()
        call("gbvlm_hbvlm_create", ctypes.cast(ctypes.pointer(h), P), len(self.verts), d, ctypes.cast(arr, PP),
             ctypes.cast(lf, P))
        self.h = h

    def __del__(self):
        try:
            if self.h:
                _lib.lib().gbvlm_hbvlm_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @staticmethod
    def _p(a):
        return ctypes.c_void_p(a.ctypes.data)

    @staticmethod
    def _colmajor(m):
        """Buffer holding the (N x N) matrix column-major (the C ABI's layout)."""
        return np.ascontiguousarray(np.asarray(m, np.float64).T)

    def prepare(self, harmonics, max_t_steps, wake_T, t_steps, times, T, Td, dft):
        self._keep = [np.ascontiguousarray(x) for x in (wake_T, T, Td)] + [self._colmajor(dft)] + \
                     [np.ascontiguousarray(t_steps, np.int64), np.ascontiguousarray(times, np.float64)]
        wT, T_, Td_, D_, ts, tm = self._keep
        call("gbvlm_hbvlm_prepare", self.h, int(harmonics), int(max_t_steps), self._p(wT), self._p(ts), self._p(tm),
             self._p(T_), self._p(Td_), self._p(D_), None)

    def map(self, x, omega, dt):
        x = np.asfortranarray(x, np.float64)
        y = np.zeros_like(x, order="F")
        call("gbvlm_hbvlm_map", self.h, self._p(x), self._p(y), float(omega), float(dt), None)
        return y

    def solve(self, x, omega, dt, max_iter, tol, m):
        it = ctypes.c_int32()
        call("gbvlm_hbvlm_solve", self.h, self._p(x), float(omega), float(dt), int(max_iter), float(tol), int(m),
             ctypes.cast(ctypes.pointer(it), P), None)
        return it.value

    def prepare_batch(self, harmonics, max_ts, wake_Ts, t_steps, times, T, Td, dfts):
        """K parameter sets: per-set wake arrays (lists), the rest stacked over the sets."""
        K = len(max_ts)
        wk = [np.ascontiguousarray(w, np.float64) for w in wake_Ts]
        keep = wk + [np.ascontiguousarray(np.asarray(max_ts, np.int64)),
                     np.ascontiguousarray(np.asarray(t_steps, np.int64)),
                     np.ascontiguousarray(np.asarray(times, np.float64)),
                     np.ascontiguousarray(np.asarray(T, np.float64)), np.ascontiguousarray(np.asarray(Td, np.float64)),
                     np.ascontiguousarray(np.stack([self._colmajor(d) for d in dfts]))]
        self._keep = keep
        mt, ts, tm, T_, Td_, D_ = keep[K:]
        wp = (ctypes.c_void_p * K)(*[w.ctypes.data for w in wk])
        call("gbvlm_hbvlm_prepare_batch", self.h, K, int(harmonics), self._p(mt), ctypes.cast(wp, PP), self._p(ts),
             self._p(tm), self._p(T_), self._p(Td_), self._p(D_), None)

    def prepare_batch_chain(self, harmonics, max_ts, chains, t_steps, times, T, Td, dfts):
        """prepare_batch with each set's wake transforms evaluated on the device from its chain parameters."""
        K = len(max_ts)
        keep = [np.ascontiguousarray(np.asarray(max_ts, np.int64)), np.ascontiguousarray(np.stack(chains)),
                np.ascontiguousarray(np.asarray(t_steps, np.int64)), np.ascontiguousarray(np.asarray(times, np.float64)),
                np.ascontiguousarray(np.asarray(T, np.float64)), np.ascontiguousarray(np.asarray(Td, np.float64)),
                np.ascontiguousarray(np.stack([self._colmajor(d) for d in dfts]))]
        self._keep = keep
        call("gbvlm_hbvlm_prepare_batch_chain", self.h, K, int(harmonics), *[self._p(a) for a in keep], None)

    def solve_batch(self, xs, omegas, dts, max_iter, tol, m):
        """xs: (K, n, N) iterates, updated in place (C-contiguous over sets, each set column-major)."""
        K = xs.shape[0]
        buf = np.ascontiguousarray(np.transpose(xs, (0, 2, 1)))  # (K, N, n): each set n x N column-major
        om = np.ascontiguousarray(omegas, np.float64)
        dt = np.ascontiguousarray(dts, np.float64)
        its = np.zeros(K, np.int32)
        call("gbvlm_hbvlm_solve_batch", self.h, K, self._p(buf), self._p(om), self._p(dt), int(max_iter), float(tol),
             int(m), self._p(its), None)
        xs[:] = np.transpose(buf, (0, 2, 1))
        return its

    def loads_batch(self, xs, dfts, ddfts, T, Td, fs, ref_a, ref_b, coupled_te, N):
        K = xs.shape[0]
        out = np.zeros((K, 3, N))
        keep = [np.ascontiguousarray(np.transpose(xs, (0, 2, 1))),
                np.ascontiguousarray(np.stack([self._colmajor(d) for d in dfts])),
                np.ascontiguousarray(np.stack([self._colmajor(d) for d in ddfts]))] + \
               [np.ascontiguousarray(a, np.float64) for a in (T, Td, fs, ref_a)]
        rb = np.ascontiguousarray(ref_b, np.float64) if ref_b is not None else None
        call("gbvlm_hbvlm_loads_batch", self.h, K, *[self._p(a) for a in keep],
             self._p(rb) if rb is not None else None, 1 if coupled_te else 0, self._p(out), None)
        return out

    def loads(self, x, dft, ddft, T, Td, fs, ref_a, ref_b, coupled_te, N):
        out = np.zeros(3 * N)
        keep = [np.asfortranarray(x, np.float64), self._colmajor(dft), self._colmajor(ddft)] + \
               [np.ascontiguousarray(a, np.float64) for a in (T, Td, fs, ref_a)]
        rb = np.ascontiguousarray(ref_b, np.float64) if ref_b is not None else None
        call("gbvlm_hbvlm_loads", self.h, *[self._p(a) for a in keep], self._p(rb) if rb is not None else None,
             1 if coupled_te else 0, self._p(out), None)
        return out.reshape(3, N)


def fourier_basis(H, omega, t):
    """The phases of ``fourier`` on the dual number (t, 1), shared by every
    coefficient row: per harmonic k, cos and sin of (t omega) k and the
    phase rate omega k."""
    out = []
    for h in range(H):
        k = float(h + 1)
        ph = (t * omega) * k
        out.append((np.cos(ph), np.sin(ph), omega * k))
    return out


def fourier_dual(row, basis, t):
    """``fourier`` on (t, 1) in closed form: value and d/dt with the
    operations of the Dual evaluation, in its order."""
    val = row[0] + 0.0 * t
    grad = np.zeros(np.shape(val))
    for h, (c, s, w) in enumerate(basis):
        val = (val + c * row[2 * h + 1]) + s * row[2 * h + 2]
        grad = (grad + (-s * w) * row[2 * h + 1]) + (c * w) * row[2 * h + 2]
    return val, grad


def _rot_y(px, a, ag):
    """rotation_matrix([px, 0, 0], [0, 1, 0], (a, ag)): the nonzero entries
    R00 = R22 = 1 - (1 - cos a), R02 = -R20 = sin a, the translation
    T0 = px - R00 px, T2 = -R20 px, and their rates."""
    s, c = np.sin(a), np.cos(a)
    sg = c * ag
    c1, c1g = 1.0 - c, 0.0 - (-s * ag)
    r00, r00g = 1.0 - c1, -c1g
    t0, t0g = px - r00 * px, 0.0 - r00g * px
    t2, t2g = 0.0 - (-s) * px, 0.0 - (-sg) * px
    return dict(r00=r00, r00g=r00g, r02=s, r02g=sg, t0=t0, t0g=t0g, t2=t2, t2g=t2g)


def _stack(e00, e02, e03, e20, e22, e23, diag):
    """(T, 4, 4) matrices with the given rows 0 and 2, row 1 = (0, diag, 0, 0), row 3 = (0, 0, 0, diag)."""
    T = np.zeros((np.size(e00), 4, 4))
    T[:, 0, 0], T[:, 0, 2], T[:, 0, 3] = e00, e02, e03
    T[:, 2, 0], T[:, 2, 2], T[:, 2, 3] = e20, e22, e23
    T[:, 1, 1] = T[:, 3, 3] = diag
    return T


def pitch_heave_series(t, sigma, heave, pitch, px, ctrl=None, qx=None):
    """Transforms and rates of the libhbvlm kinematic chain in closed form:
    free stream translation (-sigma t, 0, 0), heave (0, 0, -h), pitch about
    (px, 0, 0) and, for the flap, a control rotation about (qx, 0, 0) after
    the pitch (libhbvlm3.cpp:559-641; libhbvlm.cpp:470-515).  heave, pitch and
    ctrl are (value, rate) pairs from ``fourier_dual``.  Returns per surface
    (wing[, flap]) the (T, 4, 4) transform and rate stacks, each entry the
    value the Dual evaluation of the same chain gives."""
    d0, d0g = t * (-sigma), np.zeros_like(t) - sigma
    d2, d2g = -heave[0], -heave[1]
    P = _rot_y(px, *pitch)
    a00, a00g, a02, a02g = P["r00"], P["r00g"], P["r02"], P["r02g"]
    a03, a03g = P["t0"] + d0, P["t0g"] + d0g
    a23, a23g = P["t2"] + d2, P["t2g"] + d2g
    wing = (_stack(a00, a02, a03, -a02, a00, a23, 1.0), _stack(a00g, a02g, a03g, -a02g, a00g, a23g, 0.0))
    if ctrl is None:
        return [wing]
    B = _rot_y(qx, *ctrl)
    b00, b00g, b02, b02g = B["r00"], B["r00g"], B["r02"], B["r02g"]
    b20, b20g = -b02, -b02g
    u0, u0g, u2, u2g = B["t0"], B["t0g"], B["t2"], B["t2g"]
    rows = []
    for ar0, ar0g, ar2, ar2g, ar3, ar3g in ((a00, a00g, a02, a02g, a03, a03g), (-a02, -a02g, a00, a00g, a23, a23g)):
        m0 = ar0 * b00 + ar2 * b20
        m0g = (ar0 * b00g + ar0g * b00) + (ar2 * b20g + ar2g * b20)
        m2 = ar0 * b02 + ar2 * b00
        m2g = (ar0 * b02g + ar0g * b02) + (ar2 * b00g + ar2g * b00)
        m3 = (ar0 * u0 + ar2 * u2) + ar3
        m3g = ((ar0 * u0g + ar0g * u0) + (ar2 * u2g + ar2g * u2)) + ar3g
        rows.append((m0, m0g, m2, m2g, m3, m3g))
    (f00, f00g, f02, f02g, f03, f03g), (f20, f20g, f22, f22g, f23, f23g) = rows
    flap = (_stack(f00, f02, f03, f20, f22, f23, 1.0), _stack(f00g, f02g, f03g, f20g, f22g, f23g, 0.0))
    return [wing, flap]


class _Lazy(dict):
    """A dict whose keys in ``lazy`` are computed on first access (the host
    copies of arrays the device evaluates, kept for inspection and tests)."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.lazy = {}

    def __missing__(self, key):
        if key in self.lazy:
            self[key] = self.lazy.pop(key)()
            return self[key]
        raise KeyError(key)


def _flat_stack(series, which, sl=slice(None)):
    """(T, nsurf, 16) column-major transforms (which = 0) or rates (1) of every surface."""
    return np.stack([s[which][sl].transpose(0, 2, 1).reshape(-1, 16) for s in series], axis=1)


class _HBVLMBase:
    qc = False
    tol = 1e-12
    dt_surface = 1

    def __init__(self, backend_name, meshes, lifting):
        if backend_name not in ("gb300", "cuda", "cpu"):
            raise RuntimeError("Unsupported backend: " + backend_name)
        self.verts_raw = [read_plot3d(m, qc=self.qc).astype(np.float64) if isinstance(m, str)
                          else np.array(m, np.float64) for m in meshes]
        self.lifting = lifting
        self.m_harmonics = None

    def init(self, harmonics, scaling):
        """Scale the coordinates (libhbvlm3.cpp:176-187) and reset the coefficients."""
        self.m_harmonics = int(harmonics)
        self.m_coeffs = 2 * self.m_harmonics + 1
        self.verts = []
        for v in self.verts_raw:
            w = v.copy()
            w[:3] *= scaling
            self.verts.append(w)
        self._engine = None
        n = sum((v.shape[1] - 1) * (v.shape[2] - 1) for v in self.verts)
        self.gamma_coeffs = np.zeros((n, self.m_coeffs), order="F")

    @property
    def engine(self):
        """The device handle, created at first use (planning a run needs none)."""
        if self._engine is None:
            self._engine = HBEngine(self.verts, self.lifting)
        return self._engine

    def _chain_vector(self, S, dt):
        """k_hb_chain's parameters for set S: sigma, omega, dt, px, qx, flap, the three coefficient rows."""
        sigma, rows, px, qx, flap = self._chain_params(S)
        U = self.m_coeffs
        head = [sigma, S["omega"], dt, px, qx if qx is not None else 0.0, 1.0 if flap else 0.0]
        return np.concatenate([np.array(head)] + [np.asarray(r, np.float64) if r is not None else np.zeros(U)
                                                  for r in rows])

    def _chain_series(self, sets, own, t):
        """``_series`` for several sets at once: set own[i] at time t[i]."""
        prm = [self._chain_params(S) for S in sets]
        omega = np.array([S["omega"] for S in sets])[own]
        sigma = np.array([q[0] for q in prm])[own]
        px, qx, flap = prm[0][2], prm[0][3], prm[0][4]
        rows = [np.stack([np.asarray(q[1][r], np.float64) for q in prm], axis=-1)[:, own] for r in range(3 if flap else 2)]
        B = fourier_basis(self.m_harmonics, omega, t)
        ctrl = fourier_dual(rows[2], B, t) if flap else None
        return pitch_heave_series(t, sigma, fourier_dual(rows[0], B, t), fourier_dual(rows[1], B, t), px, ctrl, qx)

    def _series(self, S, t):
        """Transforms and rates of the surfaces' kinematic chain for parameter set S at the times t."""
        return self._chain_series([S], np.zeros(np.size(t), np.int64), np.asarray(t, np.float64))

    def plan(self, sets, refs):
        """Host side of HBVLM::run for K parameter sets (libhbvlm3.cpp:262-347):
        time step, wake length, instance and force-instance times with their
        kinematics, DFT matrices, free stream and moment reference points.
        The wake transforms of every step (``wake_T``) are computed only when
        read; the device evaluates them itself from the chain parameters."""
        N = self.m_coeffs
        chord = last_panel_chord(self.verts[self.dt_surface])
        cols, times = [], []
        for k, S in enumerate(sets):
            omega, t_start = S["omega"], S["t_start"]
            period = TWO_PI_F / omega
            interval = period / N
            if not interval > chord:
                raise AssertionError("period interval %g must exceed the last panel chord %g" % (interval, chord))
            dt = interval / math.ceil(interval / chord)
            max_t = int((t_start + period + dt) / dt)
            ts = np.array([int(round((t_start + period * q / N) / dt)) for q in range(N)], np.int64)
            fts = np.array([int(round((0.0 + period * q / N) / dt)) for q in range(N)], np.int64)
            c = _Lazy(omega=omega, dt=dt, max_t=max_t, period=period, ts=ts, tm=ts * dt, fts=fts, ftm=fts * dt)
            c.lazy["wake_T"] = (lambda S=S, c=c: _flat_stack(self._series(S, np.arange(c["max_t"]) * c["dt"]), 0))
            times += [c["tm"], c["ftm"]]
            cols.append(c)
        K = len(cols)
        own = np.repeat(np.arange(K), 2 * N)
        series = self._chain_series(sets, own, np.concatenate(times))
        for k, c in enumerate(cols):
            si, sf = slice(2 * N * k, 2 * N * k + N), slice(2 * N * k + N, 2 * N * (k + 1))
            c["inst"] = (c["ts"], c["tm"], _flat_stack(series, 0, si), _flat_stack(series, 1, si))
            c["finst"] = c["force_inst"] = (c["fts"], c["ftm"], _flat_stack(series, 0, sf), _flat_stack(series, 1, sf))
            c["dft"], c["ddft"] = dft_matrices(N, c["omega"], c["period"])
            c["fs"] = np.tile(np.array([self._chain_params(sets[k])[0], -0.0, -0.0]), (N, 1))  # -d/dt of the free stream
            c["ref_a"] = (series[0][0][sf] @ np.array([refs[0], 0.0, 0.0, 1.0]))[:, :3]
            c["ref_b"] = None
            if len(refs) > 1:
                c["ref_b"] = (series[1][0][sf] @ np.array([refs[1], 0.0, 0.0, 1.0]))[:, :3]
        return cols

    def _run_sets(self, sets, refs, forces_list, coupled_te, params=None):
        """HBVLM::run for K parameter sets (libhbvlm3.cpp:262-552), solved together.

        sets: dicts with ``omega``, ``t_start`` and the kinematic parameters
        ``_chain_params`` reads.  The wake transforms of every step are
        evaluated on the device from the chain parameters; the instances'
        transforms (2N per set) in one closed-form pass over all sets.
        Every set starts from the current coefficients, which afterwards
        hold the last set's fixed point, as after the same runs in sequence."""
        N, H = self.m_coeffs, self.m_harmonics
        cols = self.plan(sets, refs)
        K = len(cols)
        from . import autotune
        if params is not None:  # the autotuner's search sets the shapes itself
            autotune.set_params(params)
            self.tuning = {"params": dict(params), "source": "given"}
        else:
            self.tuning = autotune.apply(autotune.hbvlm_key(self.engine.n, K * N, max(c["max_t"] for c in cols),
                                                            autotune.device_sms()))
        self.engine.prepare_batch_chain(H, [c["max_t"] for c in cols],
                                  [self._chain_vector(S, c["dt"]) for S, c in zip(sets, cols)],
                                  np.concatenate([c["inst"][0] for c in cols]),
                                  np.concatenate([c["inst"][1] for c in cols]),
                                  np.concatenate([c["inst"][2] for c in cols]),
                                  np.concatenate([c["inst"][3] for c in cols]), [c["dft"] for c in cols])
        xs = np.repeat(self.gamma_coeffs[None], K, axis=0)
        its = self.engine.solve_batch(xs, [c["omega"] for c in cols], [c["dt"] for c in cols], 100, self.tol, 10)
        ref_b = np.concatenate([c["ref_b"] for c in cols]) if len(refs) > 1 else None
        out = self.engine.loads_batch(xs, [c["dft"] for c in cols], [c["ddft"] for c in cols],
                                      np.concatenate([c["finst"][2] for c in cols]),
                                      np.concatenate([c["finst"][3] for c in cols]),
                                      np.concatenate([c["fs"] for c in cols]), np.concatenate([c["ref_a"] for c in cols]),
                                      ref_b, coupled_te, N)
        for f, o in zip(forces_list, out):
            f[:, :] = o[:f.shape[0], :]
        self.gamma_coeffs[:] = xs[-1]
        self._last_batch = cols
        self._last = cols[-1]
        return its


class HBVLM3(_HBVLMBase):
    """libhbvlm3.HBVLM: wing (non-lifting) + flap (lifting), 3-DOF pitch/heave/flap."""
    qc = False
    tol = 1e-12
    dt_surface = 1
    # libhbvlm3.cpp:562-581 assigns float literals (0.127f, 52.6506f, ...) to its double fields, so the
    # kinematics use those constants rounded to float
    VARS = dict(a=float(np.float32(-0.5)), b=float(np.float32(0.127)), c=float(np.float32(0.5)),
                omega_alpha=float(np.float32(52.6506)))

    def __init__(self, backend_name, meshes):
        if len(meshes) != 2:
            raise AssertionError("libhbvlm3 expects two meshes (wing, flap)")
        super().__init__(backend_name, meshes, [False, True])

    def assembly(self, omega, U, dyn_f):
        v = self.VARS
        H = self.m_harmonics
        r = np.asarray(dyn_f, np.float64)
        tree = KinematicsTree()
        fsn = tree.add(lambda t: translation_matrix([-(U / (v["b"] * v["omega_alpha"])) * t, 0.0, 0.0]))
        heave = tree.add(lambda t: translation_matrix([0.0, 0.0, -fourier(r[0], H, omega, t)])).after(fsn)
        pitch = tree.add(lambda t: rotation_matrix([1.0 + v["a"], 0, 0], [0, 1, 0], fourier(r[1], H, omega, t))).after(heave)
        ctrl = tree.add(lambda t: rotation_matrix([1.0 + v["c"], 0, 0], [0, 1, 0], fourier(r[2], H, omega, t))).after(pitch)
        asm = Assembly(fsn)
        asm.add("wing", pitch, False)
        asm.add("flap", ctrl, True)
        return asm

    def _sigma(self, S):
        return S["U"] / (self.VARS["b"] * self.VARS["omega_alpha"])

    def _chain_params(self, S):
        """The chain of ``assembly``: free stream speed, heave / pitch / control rows, axes; the flap lifts."""
        v = self.VARS
        r = np.asarray(S["dyn"], np.float64)
        return self._sigma(S), (r[0], r[1], r[2]), 1.0 + v["a"], 1.0 + v["c"], True

    def _refs(self):
        return (1.0 + self.VARS["a"], 1.0 + self.VARS["c"])

    @staticmethod
    def parameter_set(omega, U, dyn_f):
        """One run's parameters (libhbvlm3.cpp:558-641): two cycles of wake before the period."""
        return dict(omega=omega, U=U, dyn=dyn_f, t_start=2.0 * TWO_PI_F / omega)

    def run(self, omega, U, dyn_f, forces_t):
        S = self.parameter_set(omega, U, dyn_f)
        self.iterations = int(self._run_sets([S], self._refs(), [forces_t], True)[0])
        return forces_t

    def run_batch(self, omegas, Us, dyn_fs, forces_list):
        """``run`` for K parameter sets solved together (one device solve)."""
        sets = [dict(omega=om, U=U, dyn=d, t_start=2.0 * TWO_PI_F / om) for om, U, d in zip(omegas, Us, dyn_fs)]
        self.iterations = self._run_sets(sets, self._refs(), forces_list, True)
        return forces_list


class HBVLM2(_HBVLMBase):
    """libhbvlm.HBVLM: one lifting surface, 2-DOF heave/pitch (lib/libhbvlm.cpp:470-515)."""
    qc = True
    tol = 1e-9
    dt_surface = 0
    U_INF, A_H = 1.0, -0.5

    def __init__(self, backend_name, mesh):
        super().__init__(backend_name, [mesh], [True])

    def assembly(self, omega, dyn_f):
        H = self.m_harmonics
        r = np.asarray(dyn_f, np.float64)
        u_inf, a_h = self.U_INF, self.A_H
        tree = KinematicsTree()
        fsn = tree.add(lambda t: translation_matrix([-u_inf * t, 0.0, 0.0]))
        heave = tree.add(lambda t: translation_matrix([0.0, 0.0, -fourier(r[0], H, omega, t)])).after(fsn)
        pitch = tree.add(lambda t: rotation_matrix([1.0 + a_h, 0, 0], [0, 1, 0], fourier(r[1], H, omega, t))).after(heave)
        asm = Assembly(fsn)
        asm.add("wing", pitch, True)
        return asm

    def _sigma(self, S):
        return self.U_INF

    def _chain_params(self, S):
        r = np.asarray(S["dyn"], np.float64)
        return self.U_INF, (r[0], r[1], None), 1.0 + self.A_H, None, False

    @staticmethod
    def parameter_set(omega, dyn_f):
        """One run's parameters (libhbvlm.cpp:470-515): three cycles of wake before the period."""
        return dict(omega=omega, dyn=dyn_f, t_start=3.0 * TWO_PI_F / omega)

    def run(self, omega, dyn_f, forces_t):
        S = self.parameter_set(omega, dyn_f)
        self.iterations = int(self._run_sets([S], (0.5,), [forces_t], False)[0])
        return forces_t

    def run_batch(self, omegas, dyn_fs, forces_list):
        """``run`` for K parameter sets solved together (one device solve)."""
        sets = [dict(omega=om, dyn=d, t_start=3.0 * TWO_PI_F / om) for om, d in zip(omegas, dyn_fs)]
        self.iterations = self._run_sets(sets, (0.5,), forces_list, False)
        return forces_list
