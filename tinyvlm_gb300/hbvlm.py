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


def hb_arrays(assembly, N, dt, max_t_steps, t_start, period):
    """Wake transforms per step, instance transforms/rates for the map and for the loads."""
    nodes = assembly.surface_kinematics()
    ns = len(nodes)
    wake_T = np.zeros((max_t_steps, ns, 16))
    tw = np.arange(max_t_steps) * dt
    for m, nd in enumerate(nodes):
        v, _ = nd.transform_series(tw)
        wake_T[:, m] = v.transpose(0, 2, 1).reshape(-1, 16)

    def inst(start):
        ts = np.array([int(round((start + period * s / N) / dt)) for s in range(N)], np.int64)
        tm = ts * dt
        T = np.zeros((N, ns, 16))
        Td = np.zeros((N, ns, 16))
        for m, nd in enumerate(nodes):
            v, d = nd.transform_series(tm)
            T[:, m] = v.transpose(0, 2, 1).reshape(-1, 16)
            Td[:, m] = d.transpose(0, 2, 1).reshape(-1, 16)
        return ts, tm, T, Td

    return wake_T, inst(t_start), inst(0.0)


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
        self.engine = HBEngine(self.verts, self.lifting)
        self.gamma_coeffs = np.zeros((self.engine.n, self.m_coeffs), order="F")

    def _run(self, t_start, omega, assembly, refs, forces_t, coupled_te):
        N, H = self.m_coeffs, self.m_harmonics
        period = TWO_PI_F / omega
        interval = period / N
        chord = last_panel_chord(self.verts[self.dt_surface])
        if not interval > chord:
            raise AssertionError("period interval %g must exceed the last panel chord %g" % (interval, chord))
        dt = interval / math.ceil(interval / chord)
        max_t = int((t_start + period + dt) / dt)
        wake_T, (ts, tm, T, Td), (fts, ftm, fT, fTd) = hb_arrays(assembly, N, dt, max_t, t_start, period)
        dft, ddft = dft_matrices(N, omega, period)
        self.engine.prepare(H, max_t, wake_T, ts, tm, T, Td, dft)
        self.iterations = self.engine.solve(self.gamma_coeffs, omega, dt, 100, self.tol, 10)
        _, da = assembly.kinematics().transform_series(ftm)
        fs = -da[:, :3, 3]
        v0, _ = assembly.surface_kinematics()[0].transform_series(ftm)
        ref_a = (v0 @ np.array([refs[0], 0.0, 0.0, 1.0]))[:, :3]
        ref_b = None
        if len(refs) > 1:
            v1, _ = assembly.surface_kinematics()[1].transform_series(ftm)
            ref_b = (v1 @ np.array([refs[1], 0.0, 0.0, 1.0]))[:, :3]
        out = self.engine.loads(self.gamma_coeffs, dft, ddft, fT, fTd, fs, ref_a, ref_b, coupled_te, N)
        rows = forces_t.shape[0]
        forces_t[:, :] = out[:rows, :]
        self._last = dict(dt=dt, max_t=max_t, period=period, wake_T=wake_T, inst=(ts, tm, T, Td),
                          force_inst=(fts, ftm, fT, fTd), dft=dft, ddft=ddft, fs=fs, ref_a=ref_a, ref_b=ref_b)
        return forces_t


    def _run_batch(self, t_starts, omegas, assemblies, refs, forces_list, coupled_te):
        """Every parameter set starts from the current coefficients; afterwards
        they hold the last set's fixed point, as after the same runs in sequence."""
        N, H = self.m_coeffs, self.m_harmonics
        chord = last_panel_chord(self.verts[self.dt_surface])
        K = len(omegas)
        cols = []
        for t_start, omega, asm in zip(t_starts, omegas, assemblies):
            period = TWO_PI_F / omega
            interval = period / N
            if not interval > chord:
                raise AssertionError("period interval %g must exceed the last panel chord %g" % (interval, chord))
            dt = interval / math.ceil(interval / chord)
            max_t = int((t_start + period + dt) / dt)
            wake_T, inst, finst = hb_arrays(asm, N, dt, max_t, t_start, period)
            dft, ddft = dft_matrices(N, omega, period)
            _, da = asm.kinematics().transform_series(finst[1])
            fs = -da[:, :3, 3]
            v0, _ = asm.surface_kinematics()[0].transform_series(finst[1])
            ref_a = (v0 @ np.array([refs[0], 0.0, 0.0, 1.0]))[:, :3]
            ref_b = None
            if len(refs) > 1:
                v1, _ = asm.surface_kinematics()[1].transform_series(finst[1])
                ref_b = (v1 @ np.array([refs[1], 0.0, 0.0, 1.0]))[:, :3]
            cols.append(dict(dt=dt, max_t=max_t, wake_T=wake_T, inst=inst, finst=finst, dft=dft, ddft=ddft, fs=fs,
                             ref_a=ref_a, ref_b=ref_b))
        self.engine.prepare_batch(H, [c["max_t"] for c in cols], [c["wake_T"] for c in cols],
                                  np.concatenate([c["inst"][0] for c in cols]),
                                  np.concatenate([c["inst"][1] for c in cols]),
                                  np.concatenate([c["inst"][2] for c in cols]),
                                  np.concatenate([c["inst"][3] for c in cols]), [c["dft"] for c in cols])
        xs = np.repeat(self.gamma_coeffs[None], K, axis=0)
        self.iterations = self.engine.solve_batch(xs, omegas, [c["dt"] for c in cols], 100, self.tol, 10)
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
        return forces_list


class HBVLM3(_HBVLMBase):
    """libhbvlm3.HBVLM: wing (non-lifting) + flap (lifting), 3-DOF pitch/heave/flap."""
    qc = False
    tol = 1e-12
    dt_surface = 1
    VARS = dict(a=-0.5, b=0.127, c=0.5, omega_alpha=52.6506)

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

    def run(self, omega, U, dyn_f, forces_t):
        t_final = 2.0 * TWO_PI_F / omega
        asm = self.assembly(omega, U, dyn_f)
        return self._run(t_final, omega, asm, (1.0 + self.VARS["a"], 1.0 + self.VARS["c"]), forces_t, True)

    def run_batch(self, omegas, Us, dyn_fs, forces_list):
        """``run`` for K parameter sets solved together (one device solve)."""
        asms = [self.assembly(om, U, d) for om, U, d in zip(omegas, Us, dyn_fs)]
        return self._run_batch([2.0 * TWO_PI_F / om for om in omegas], list(omegas), asms,
                               (1.0 + self.VARS["a"], 1.0 + self.VARS["c"]), forces_list, True)


class HBVLM2(_HBVLMBase):
    """libhbvlm.HBVLM: one lifting surface, 2-DOF heave/pitch (lib/libhbvlm.cpp:470-515)."""
    qc = True
    tol = 1e-9
    dt_surface = 0

    def __init__(self, backend_name, mesh):
        super().__init__(backend_name, [mesh], [True])

    def assembly(self, omega, dyn_f):
        H = self.m_harmonics
        r = np.asarray(dyn_f, np.float64)
        u_inf, a_h = 1.0, -0.5
        tree = KinematicsTree()
        fsn = tree.add(lambda t: translation_matrix([-u_inf * t, 0.0, 0.0]))
        heave = tree.add(lambda t: translation_matrix([0.0, 0.0, -fourier(r[0], H, omega, t)])).after(fsn)
        pitch = tree.add(lambda t: rotation_matrix([1.0 + a_h, 0, 0], [0, 1, 0], fourier(r[1], H, omega, t))).after(heave)
        asm = Assembly(fsn)
        asm.add("wing", pitch, True)
        return asm

    def run(self, omega, dyn_f, forces_t):
        t_final = 3.0 * TWO_PI_F / omega
        asm = self.assembly(omega, dyn_f)
        return self._run(t_final, omega, asm, (0.5,), forces_t, False)

    def run_batch(self, omegas, dyn_fs, forces_list):
        """``run`` for K parameter sets solved together (one device solve)."""
        asms = [self.assembly(om, d) for om, d in zip(omegas, dyn_fs)]
        return self._run_batch([3.0 * TWO_PI_F / om for om in omegas], list(omegas), asms, (0.5,), forces_list,
                               False)
