"""2dtissue_gb300 — GB300-native per-step active-particle update of 2DTissue.

Thin Python harness over the C-ABI in include/tds.h (ctypes). The package name starts with a
digit, so import it with ``importlib.import_module("2dtissue_gb300")``.

Objects:
  Mesh        closed surface + unit-square UV chart (icosphere ellipsoid, bumpy sphere, OFF file)
  Simulation  one system (R = 1) or a ragged ensemble of replicas on one mesh
  Tissue      the reference's _2DTissue interface: start(), update(), is_finished(),
              get_order_parameter() (src/simulation/2DTissue.h:37-60)

The CUDA library is required: every simulation call fails loudly (RuntimeError) when the
extension is missing or there is no GPU. There is no CPU fallback.
"""
import ctypes as C
import os
from dataclasses import dataclass, asdict

import numpy as np

from . import build as _build

TDS_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error / no CUDA device", 3: "mesh error", 4: "device status set",
          5: "out of device memory", 6: "size limit"}
STATUS_BITS = {1: "non-finite", 2: "wrap limit", 4: "locate fallback", 16: "particle outside the surface cells"}

_lib = None


class TdsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("tds error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


class _Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("radius", "k_rep", "k_adh", "r_max", "v0", "mu", "tau", "align",
                                          "eta", "dt")] + [("force_mode", C.c_int), ("reserved", C.c_int)]


class _AdjSpec(C.Structure):
    _fields_ = [("n_steps", C.c_int), ("checkpoint_stride", C.c_int), ("r3d_target", C.c_void_p),
                ("w_pos", C.c_double), ("phi_target", C.c_void_p), ("w_phi", C.c_double), ("window", C.c_int),
                ("gather_lanes", C.c_int)]


class _AdjResult(C.Structure):
    _fields_ = [("loss", C.c_double), ("d_params", C.c_void_p), ("d_uv0", C.c_void_p), ("d_theta0", C.c_void_p),
                ("checkpoint_stride", C.c_int)]


# the reference's Particle record (src/simulation/Struct.h:9-29) as tds_get_particles fills it
PARTICLE_DTYPE = np.dtype({"names": ["x_UV", "y_UV", "x_velocity_UV", "y_velocity_UV", "alignment_UV",
                                     "compass_north_pole_UV", "compass_south_pole_UV", "x_3D", "y_3D", "z_3D",
                                     "neighbor_count"],
                           "formats": ["<f8"] * 10 + ["<i4"],
                           "offsets": [8 * k for k in range(10)] + [80], "itemsize": 88})

# order of the parameter gradients returned by the adjoint
GRAD_PARAMS = ("k_rep", "k_adh", "v0", "mu", "tau", "align", "eta")


class _Tuning(C.Structure):
    _fields_ = [("cells_per_particle", C.c_double), ("step_block", C.c_int), ("graph_steps", C.c_int),
                ("lanes_per_particle", C.c_int)]


class _RefParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("v0", "k", "sigma", "r_adh", "k_adh", "step_size")]


class _StateView(C.Structure):
    _fields_ = [("uv", C.c_void_p), ("theta", C.c_void_p), ("face", C.c_void_p), ("r3d", C.c_void_p),
                ("vel_uv", C.c_void_p), ("nbr_count", C.c_void_p)]


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Loads (building if needed) the in-tree CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("lib2dtissue_gb300.so is not built (run __graft_entry__.build())")
        _build.build()
    L = C.CDLL(path)
    P, I, D, VP = C.POINTER, C.c_int, C.c_double, C.c_void_p
    L.tds_mesh_ellipsoid.argtypes = [I, D, D, D, P(VP)]
    L.tds_mesh_bumpy_sphere.argtypes = [I, D, D, P(VP)]
    L.tds_mesh_from_arrays.argtypes = [VP, I, VP, I, P(VP)]
    L.tds_mesh_load_off.argtypes = [C.c_char_p, P(VP)]
    L.tds_mesh_save_off.argtypes = [VP, C.c_char_p]
    L.tds_mesh_info.argtypes = [VP, P(I), P(I), P(I), P(D)]
    L.tds_mesh_arrays.argtypes = [VP, VP, VP, VP, VP, VP]
    L.tds_mesh_destroy.argtypes = [VP]
    L.tds_mesh_last_error.restype = C.c_char_p
    L.tds_create.argtypes = [VP, P(_Params), I, C.c_uint64, I, P(VP)]
    L.tds_ensemble_create.argtypes = [VP, I, VP, VP, C.c_uint64, I, P(VP)]
    L.tds_start.argtypes = [VP]
    L.tds_step.argtypes = [VP, I, VP]
    L.tds_update.argtypes = [VP, P(_StateView)]
    L.tds_set_state.argtypes = [VP, P(_StateView)]
    L.tds_get_state.argtypes = [VP, P(_StateView)]
    L.tds_get_state_noalloc.argtypes = [VP, P(_StateView)]
    L.tds_get_particles.argtypes = [VP, VP]
    L.tds_step_neighbors.argtypes = [VP, I, VP]
    L.tds_set_state_async.argtypes = [VP, P(_StateView)]
    L.tds_get_state_async.argtypes = [VP, P(_StateView)]
    # tds_state_view_f32 has the same layout (six pointers)
    for name in ("tds_set_state_f32", "tds_get_state_f32", "tds_set_state_f32_async", "tds_get_state_f32_async"):
        getattr(L, name).argtypes = [VP, P(_StateView)]
    L.tds_sync.argtypes = [VP]
    L.tds_set_params.argtypes = [VP, VP]
    L.tds_create_ex.argtypes = [VP, I, VP, VP, C.c_uint64, I, P(_Tuning), P(VP)]
    L.tds_get_tuning.argtypes = [VP, P(_Tuning)]
    L.tds_autotune.argtypes = [VP, I, VP, VP, C.c_uint64, I, I, P(_Tuning), P(D)]
    L.tds_adjoint_run.argtypes = [VP, P(_AdjSpec), P(_AdjResult)]
    L.tds_adjoint_release.argtypes = [VP]
    L.tds_get_order_parameter.argtypes = [VP, VP, VP, I, P(I)]
    L.tds_get_step.argtypes = [VP, P(C.c_int64)]
    L.tds_get_status.argtypes = [VP, P(I)]
    L.tds_clear_status.argtypes = [VP]
    L.tds_num_particles.argtypes = [VP, P(I), P(I)]
    L.tds_stream.argtypes = [VP, P(VP)]
    L.tds_step_async.argtypes = [VP, I]
    L.tds_kernel_timing.argtypes = [VP, I]
    L.tds_kernel_times.argtypes = [VP, VP, VP]
    L.tds_kernels_per_step.argtypes = [VP, P(I)]
    L.tds_last_error.argtypes = [VP]
    L.tds_last_error.restype = C.c_char_p
    L.tds_destroy.argtypes = [VP]
    L.tds_debug_seam_wrap.argtypes = [I, VP, VP, VP, VP, VP, I]
    L.tds_ref_vertex_distances.argtypes = [VP, VP]
    L.tds_ref_create.argtypes = [VP, VP, P(_RefParams), I, C.c_uint64, P(VP)]
    L.tds_ref_start.argtypes = [VP]
    L.tds_ref_set_state.argtypes = [VP, VP, VP, VP]
    L.tds_ref_step.argtypes = [VP, I]
    L.tds_ref_get_state.argtypes = [VP, VP, VP, VP, VP, VP, VP]
    L.tds_ref_get_order_parameter.argtypes = [VP, VP, I, P(I)]
    L.tds_ref_stream.argtypes = [VP, P(VP)]
    L.tds_ref_last_error.argtypes = [VP]
    L.tds_ref_last_error.restype = C.c_char_p
    L.tds_ref_destroy.argtypes = [VP]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


@dataclass
class Params:
    """Model parameters; defaults are those of the 100-particle (2,1,1)-ellipsoid system (radius 0.05, r_max = 2.4 R)."""
    radius: float = 0.05
    k_rep: float = 10.0
    k_adh: float = 0.75
    r_max: float = 0.12
    v0: float = 1.0
    mu: float = 1.0
    tau: float = 1.0
    align: float = 0.5
    eta: float = 0.5
    dt: float = 0.02
    force_mode: int = 0

    def to_c(self):
        p = _Params()
        for k, v in asdict(self).items():
            setattr(p, k, v)
        return p

    def oracle_dict(self):
        return dict(R=self.radius, k=self.k_rep, k_adh=self.k_adh, r_max=self.r_max, v0=self.v0, mu=self.mu,
                    tau=self.tau, align=self.align, eta=self.eta, dt=self.dt)


class Mesh:
    """Closed triangulated surface with its unit-square UV chart."""

    def __init__(self, handle):
        self.h = C.c_void_p(handle)
        V, F, Vuv, A = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        lib().tds_mesh_info(self.h, C.byref(V), C.byref(F), C.byref(Vuv), C.byref(A))
        self.V, self.F, self.Vuv, self.area = V.value, F.value, Vuv.value, A.value

    @staticmethod
    def _make(fn, *args):
        h = C.c_void_p()
        rc = fn(*args, C.byref(h))
        if rc != TDS_OK:
            raise TdsError(rc, lib().tds_mesh_last_error().decode())
        return Mesh(h.value)

    @classmethod
    def ellipsoid(cls, level, axes=(1.0, 1.0, 1.0)):
        return cls._make(lib().tds_mesh_ellipsoid, int(level), *map(float, axes))

    @classmethod
    def bumpy_sphere(cls, level, amp=0.2, scale=5.0):
        return cls._make(lib().tds_mesh_bumpy_sphere, int(level), float(amp), float(scale))

    @classmethod
    def from_arrays(cls, v3, f3):
        v3 = np.ascontiguousarray(v3, np.float64)
        f3 = np.ascontiguousarray(f3, np.int32)
        return cls._make(lib().tds_mesh_from_arrays, v3.ctypes.data, len(v3), f3.ctypes.data, len(f3))

    @classmethod
    def load_off(cls, path):
        return cls._make(lib().tds_mesh_load_off, os.fsencode(path))

    def save_off(self, path):
        rc = lib().tds_mesh_save_off(self.h, os.fsencode(path))
        if rc:
            raise TdsError(rc, lib().tds_mesh_last_error().decode())

    def arrays(self):
        v3 = np.zeros((self.V, 3))
        f3 = np.zeros((self.F, 3), np.int32)
        uv = np.zeros((self.Vuv, 2))
        fuv = np.zeros((self.F, 3), np.int32)
        uv2v = np.zeros(self.Vuv, np.int32)
        lib().tds_mesh_arrays(self.h, v3.ctypes.data, f3.ctypes.data, uv.ctypes.data, fuv.ctypes.data,
                              uv2v.ctypes.data)
        return dict(v3=v3, f3=f3, uv=uv, fuv=fuv, uv2v=uv2v)

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.tds_mesh_destroy(self.h)
            self.h = None


class Simulation:
    """One system (n_particles int) or a ragged ensemble (n_particles list, params list)."""

    def __init__(self, mesh, params, n_particles, seed=0, precision=32, tuning=None):
        self.mesh = mesh
        self._pending = []  # host arrays of enqueued transfers, held until sync()
        L = lib()
        h = C.c_void_p()
        if tuning is not None:
            n = np.atleast_1d(np.ascontiguousarray(n_particles, np.int32))
            ps = list(params) if isinstance(params, (list, tuple)) else [params] * len(n)
            self.params = ps
            arr = (_Params * len(n))(*[q.to_c() for q in ps])
            t = _Tuning(float(tuning["cells_per_particle"]), int(tuning["step_block"]), int(tuning["graph_steps"]),
                        int(tuning.get("lanes_per_particle", 1)))
            rc = L.tds_create_ex(mesh.h, len(n), n.ctypes.data, C.cast(arr, C.c_void_p), C.c_uint64(seed),
                                 int(precision), C.byref(t), C.byref(h))
        elif np.ndim(n_particles) == 0:
            self.params = [params]
            p = params.to_c()
            rc = L.tds_create(mesh.h, C.byref(p), int(n_particles), C.c_uint64(seed), int(precision), C.byref(h))
        else:
            n = np.ascontiguousarray(n_particles, np.int32)
            ps = list(params) if isinstance(params, (list, tuple)) else [params] * len(n)
            self.params = ps
            arr = (_Params * len(n))(*[q.to_c() for q in ps])
            rc = L.tds_ensemble_create(mesh.h, len(n), n.ctypes.data, C.cast(arr, C.c_void_p), C.c_uint64(seed),
                                       int(precision), C.byref(h))
        if rc != TDS_OK:
            raise TdsError(rc, "create failed (no CUDA device, bad parameters or size limit)")
        self.h = h
        nt, nr = C.c_int(), C.c_int()
        L.tds_num_particles(self.h, C.byref(nt), C.byref(nr))
        self.N, self.R = nt.value, nr.value
        self.precision = precision
        self.seed = seed

    def _check(self, rc):
        if rc != TDS_OK:
            raise TdsError(rc, lib().tds_last_error(self.h).decode())

    def start(self):
        self._check(lib().tds_start(self.h))

    def step(self, n=1, noise=None):
        nz = None if noise is None else np.ascontiguousarray(noise, np.float64)
        if nz is not None and nz.size != n * self.N:
            raise ValueError("noise must have n_steps * N entries")
        self._check(lib().tds_step(self.h, int(n), _ptr(nz)))

    def step_async(self, n=1):
        """Launches n steps without waiting (status checked by the next step() / status())."""
        self._check(lib().tds_step_async(self.h, int(n)))

    def kernel_timing(self, enable=True):
        self._check(lib().tds_kernel_timing(self.h, int(bool(enable))))

    def kernel_times(self):
        """{name: (total_ms, launches)} for scan, scatter, order, step, finalize."""
        ms = np.zeros(5)
        n = np.zeros(5, np.int64)
        self._check(lib().tds_kernel_times(self.h, ms.ctypes.data, n.ctypes.data))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(("scan", "scatter", "order", "step", "finalize"))}

    # State transfers. Float arrays are float64 (tds_state_view) or, for an FP32 handle, float32
    # (tds_state_view_f32: the device values as they are, half the bytes over the host link).
    def _in_view(self, uv, theta, face, r3d):
        ft = np.float32 if np.asarray(uv).dtype == np.float32 else np.float64
        uv = np.ascontiguousarray(uv, ft)
        th = np.ascontiguousarray(theta, ft)
        fc = None if face is None else np.ascontiguousarray(face, np.int32)
        r3 = None if r3d is None else np.ascontiguousarray(r3d, ft)
        return ft == np.float32, (uv, th, fc, r3), _StateView(_ptr(uv), _ptr(th), _ptr(fc), _ptr(r3), None, None)

    def _out_view(self, out, who):
        fl = [out[k] for k in ("uv", "theta", "r3d", "vel_uv") if out.get(k) is not None]
        ft = fl[0].dtype if fl else np.dtype(np.float64)
        if ft not in (np.float32, np.float64):
            raise ValueError("%s: float arrays must be float64 or float32" % who)
        for k, dt, per in (("uv", ft, 2), ("theta", ft, 1), ("face", np.int32, 1), ("r3d", ft, 3),
                           ("vel_uv", ft, 2), ("nbr", np.int32, 1)):
            a = out.get(k)
            if a is not None and not (a.flags.c_contiguous and a.dtype == dt and a.size == per * self.N):
                raise ValueError("%s: out[%r] must be a C-contiguous %s array of %d values"
                                 % (who, k, np.dtype(dt).name, per * self.N))
        v = _StateView(_ptr(out.get("uv")), _ptr(out.get("theta")), _ptr(out.get("face")), _ptr(out.get("r3d")),
                       _ptr(out.get("vel_uv")), _ptr(out.get("nbr")))
        return ft == np.float32, v

    def set_state(self, uv, theta, face=None, r3d=None):
        f32, _, v = self._in_view(uv, theta, face, r3d)
        self._check((lib().tds_set_state_f32 if f32 else lib().tds_set_state)(self.h, C.byref(v)))

    def get_state(self, out=None, dtype=np.float64):
        N = self.N
        o = out if out is not None else dict(uv=np.zeros((N, 2), dtype), theta=np.zeros(N, dtype),
                                            face=np.zeros(N, np.int32), r3d=np.zeros((N, 3), dtype),
                                            vel_uv=np.zeros((N, 2), dtype), nbr=np.zeros(N, np.int32))
        f32, v = self._out_view(o, "get_state")
        self._check((lib().tds_get_state_f32 if f32 else lib().tds_get_state)(self.h, C.byref(v)))
        return o

    def set_state_async(self, uv, theta, face=None, r3d=None):
        """Enqueues set_state (upload stream + load on the compute stream) and returns; the
        arrays are held until sync()."""
        f32, arrays, v = self._in_view(uv, theta, face, r3d)
        self._pending.append(arrays)
        self._check((lib().tds_set_state_f32_async if f32 else lib().tds_set_state_async)(self.h, C.byref(v)))

    def get_state_async(self, out):
        """Enqueues get_state into the preallocated arrays of `out` (gather on the compute
        stream, download stream for the copies); they are valid after sync()."""
        f32, v = self._out_view(out, "get_state_async")
        self._pending.append(out)
        self._check((lib().tds_get_state_f32_async if f32 else lib().tds_get_state_async)(self.h, C.byref(v)))

    def sync(self):
        """Waits for everything enqueued on this handle; raises on a non-zero device status."""
        try:
            self._check(lib().tds_sync(self.h))
        finally:
            self._pending = []

    def tuning(self):
        t = _Tuning()
        self._check(lib().tds_get_tuning(self.h, C.byref(t)))
        return dict(cells_per_particle=t.cells_per_particle, step_block=t.step_block, graph_steps=t.graph_steps,
                    lanes_per_particle=t.lanes_per_particle)

    def set_params(self, params):
        """New model parameters (one Params, or one per replica); radius and r_max must not change."""
        ps = list(params) if isinstance(params, (list, tuple)) else [params] * self.R
        arr = (_Params * len(ps))(*[q.to_c() for q in ps])
        self._check(lib().tds_set_params(self.h, C.cast(arr, C.c_void_p)))
        self.params = ps

    def adjoint(self, n_steps, r3d_target=None, w_pos=0.0, phi_target=None, w_phi=0.0, checkpoint_stride=0,
                window=0, gather_lanes=0):
        """Runs n_steps forward from the current state, then the hand-written reverse sweep.
        Loss = w_pos * sum_r mean_i |r_T - r*|^2 + w_phi * sum_t sum_r (phi_t - phi*_t)^2.
        Returns loss, d_params (R x 7, order GRAD_PARAMS), d_uv0 (N x 2), d_theta0 (N) and the
        checkpoint stride used. window (0 < window < n_steps): truncated gradient over the last
        `window` steps; d_uv0 / d_theta0 are then with respect to the state at the window's start.
        gather_lanes: lanes per particle of the reverse neighbour gather (0 = by system size, 1, 4)."""
        N, R = self.N, self.R
        tgt = None if r3d_target is None else np.ascontiguousarray(r3d_target, np.float64).reshape(N, 3)
        phi = None if phi_target is None else np.ascontiguousarray(phi_target, np.float64).reshape(n_steps, R)
        spec = _AdjSpec(int(n_steps), int(checkpoint_stride), _ptr(tgt), float(w_pos), _ptr(phi), float(w_phi),
                        int(window), int(gather_lanes))
        dp = np.zeros((R, 8))
        duv = np.empty((N, 2))  # written in full by the library
        dth = np.empty(N)
        res = _AdjResult(0.0, _ptr(dp), _ptr(duv), _ptr(dth), 0)
        self._check(lib().tds_adjoint_run(self.h, C.byref(spec), C.byref(res)))
        return dict(loss=res.loss, d_params=dp[:, :7], d_uv0=duv, d_theta0=dth, checkpoint_stride=res.checkpoint_stride)

    def adjoint_release(self):
        """Frees the adjoint's work memory that the handle keeps between adjoint() calls."""
        self._check(lib().tds_adjoint_release(self.h))

    def step_neighbors(self, cap=64):
        """One step that also returns the neighbours it used: (N, cap) int32, row i the indices of
        particle i's neighbours in the step's visiting order, -1 past the last (test hook)."""
        out = np.full((self.N, int(cap)), -1, np.int32)
        self._check(lib().tds_step_neighbors(self.h, int(cap), out.ctypes.data))
        return out

    def get_particles(self):
        """update()'s Particle records (numpy structured array, PARTICLE_DTYPE), packed on the device."""
        out = np.zeros(self.N, PARTICLE_DTYPE)
        self._check(lib().tds_get_particles(self.h, out.ctypes.data))
        return out

    def get_state_noalloc(self, out=None):
        """Same as get_state, staged in the library's fixed device array (no device allocation;
        at most 233,016 particles; calls that overlap on the GPU race)."""
        N = self.N
        o = out if out is not None else dict(uv=np.zeros((N, 2)), theta=np.zeros(N), face=np.zeros(N, np.int32),
                                            r3d=np.zeros((N, 3)), vel_uv=np.zeros((N, 2)),
                                            nbr=np.zeros(N, np.int32))
        # the entry point fills double arrays of N values per component; any array passed is
        # checked for type, size and layout before the library writes into it (absent keys are
        # not read back)
        f32, v = self._out_view(o, "get_state_noalloc")
        if f32:
            raise ValueError("get_state_noalloc: float arrays must be float64 (the entry point fills double arrays)")
        self._check(lib().tds_get_state_noalloc(self.h, C.byref(v)))
        return o

    def order_parameter(self):
        n = C.c_int()
        lib().tds_get_order_parameter(self.h, None, None, 0, C.byref(n))
        phi = np.zeros(n.value * self.R)
        psi = np.zeros(n.value * self.R)
        self._check(lib().tds_get_order_parameter(self.h, phi.ctypes.data, psi.ctypes.data, len(phi), C.byref(n)))
        return phi.reshape(n.value, self.R), psi.reshape(n.value, self.R)

    @property
    def step_count(self):
        s = C.c_int64()
        lib().tds_get_step(self.h, C.byref(s))
        return s.value

    def status(self):
        s = C.c_int()
        self._check(lib().tds_get_status(self.h, C.byref(s)))
        return s.value

    def clear_status(self):
        self._check(lib().tds_clear_status(self.h))

    def stream(self):
        p = C.c_void_p()
        self._check(lib().tds_stream(self.h, C.byref(p)))
        return p.value

    def kernels_per_step(self):
        n = C.c_int()
        self._check(lib().tds_kernels_per_step(self.h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.tds_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Tissue:
    """The reference facade (_2DTissue, src/simulation/2DTissue.h:37-60) over the GPU step.

    Argument meaning follows the reference ctor: sigma is the particle radius, r_adh the
    interaction cut-off, step_size the time step. The reference's CLI passes --step-time into
    the v0 slot (main.cpp:76-84); here step_size is the time step, stated explicitly.
    """

    def __init__(self, save_data=False, particle_innenleben=False, free_boundary=False, mesh_path=None,
                 particle_count=1000, step_count=1, v0=0.1, use_kafka=False, k=1.0, k_next=10.0, v0_next=0.1,
                 sigma=0.4166666666666667, mu=1.0, r_adh=1.0, k_adh=0.75, step_size=0.001, map_cache_count=30,
                 tau=1.0, align=0.5, eta=0.0, seed=0, precision=32, mesh=None):
        self.mesh = mesh if mesh is not None else (Mesh.load_off(mesh_path) if mesh_path else Mesh.ellipsoid(4, (2, 1, 1)))
        self.params = Params(radius=sigma, k_rep=k, k_adh=k_adh, r_max=r_adh, v0=v0, mu=mu, tau=tau, align=align,
                             eta=eta, dt=step_size)
        self.step_count = int(step_count)
        self.current_step = 0
        self.sim = Simulation(self.mesh, self.params, int(particle_count), seed=seed, precision=precision)

    def start(self):
        self.sim.start()

    def update(self):
        """One step; returns the System record: order parameter + per-particle arrays."""
        self.sim.step(1)
        self.current_step += 1
        st = self.sim.get_state()
        phi, _ = self.sim.order_parameter()
        return dict(order_parameter=float(phi[-1, 0]), particles=st)

    def is_finished(self):
        return self.current_step >= self.step_count

    def get_order_parameter(self):
        phi, _ = self.sim.order_parameter()
        return phi[:, 0]


@dataclass
class RefParams:
    """Parameters of the reference-semantics step: the _2DTissue ctor defaults (2DTissue.h:37-54)."""
    v0: float = 0.1
    k: float = 1.0
    sigma: float = 0.41667
    r_adh: float = 1.0
    k_adh: float = 0.75
    step_size: float = 0.001

    def to_c(self):
        return _RefParams(*[float(v) for v in asdict(self).values()])


def ref_vertex_distances(mesh):
    """Chart-vertex distance matrix (shortest paths along mesh edges), Vuv x Vuv."""
    out = np.zeros((mesh.Vuv, mesh.Vuv))
    rc = lib().tds_ref_vertex_distances(mesh.h, out.ctypes.data)
    if rc != TDS_OK:
        raise TdsError(rc, "vertex distances failed")
    return out


class RefSimulation:
    """The reference's own step on the device (FP64): integer-degree polarity, vertex-snapped pair
    distances from a dense matrix, chart-difference forces, brute-force face search
    (tds_ref_* in include/tds.h)."""

    def __init__(self, mesh, params, n_particles, seed=0, vertex_dist=None):
        self.mesh = mesh
        self.N = int(n_particles)
        D = None if vertex_dist is None else np.ascontiguousarray(vertex_dist, np.float64)
        if D is not None and D.shape != (mesh.Vuv, mesh.Vuv):
            raise ValueError("vertex_dist must be Vuv x Vuv")
        h = C.c_void_p()
        p = params.to_c()
        rc = lib().tds_ref_create(mesh.h, _ptr(D), C.byref(p), self.N, C.c_uint64(seed), C.byref(h))
        if rc != TDS_OK:
            raise TdsError(rc, "ref create failed (no CUDA device, bad parameters or size limit)")
        self.h = h

    def _check(self, rc):
        if rc != TDS_OK:
            raise TdsError(rc, lib().tds_ref_last_error(self.h).decode())

    def start(self):
        self._check(lib().tds_ref_start(self.h))

    def set_state(self, r_uv, n_deg, nearest=None):
        u = np.ascontiguousarray(r_uv, np.float64)
        n = np.ascontiguousarray(n_deg, np.int32)
        nv = None if nearest is None else np.ascontiguousarray(nearest, np.int32)
        self._check(lib().tds_ref_set_state(self.h, u.ctypes.data, n.ctypes.data, _ptr(nv)))

    def step(self, n=1):
        self._check(lib().tds_ref_step(self.h, int(n)))

    def get_state(self):
        N = self.N
        out = dict(uv=np.zeros((N, 2)), n_deg=np.zeros(N, np.int32), nearest=np.zeros(N, np.int32),
                   r3d=np.zeros((N, 3)), r_dot=np.zeros((N, 2)), nbr=np.zeros(N, np.int32))
        self._check(lib().tds_ref_get_state(self.h, *[out[k].ctypes.data for k in
                                                      ("uv", "n_deg", "nearest", "r3d", "r_dot", "nbr")]))
        return out

    def order_parameter(self):
        n = C.c_int()
        self._check(lib().tds_ref_get_order_parameter(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        self._check(lib().tds_ref_get_order_parameter(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def stream(self):
        s = C.c_void_p()
        self._check(lib().tds_ref_stream(self.h, C.byref(s)))
        return s.value

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.tds_ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def autotune(mesh, params, n_particles, seed=0, precision=32, trial_steps=64):
    """Times each candidate tuning on this workload; returns (tuning dict, particle-steps/s)."""
    n = np.atleast_1d(np.ascontiguousarray(n_particles, np.int32))
    ps = list(params) if isinstance(params, (list, tuple)) else [params] * len(n)
    arr = (_Params * len(n))(*[q.to_c() for q in ps])
    t, rate = _Tuning(), C.c_double()
    rc = lib().tds_autotune(mesh.h, len(n), n.ctypes.data, C.cast(arr, C.c_void_p), C.c_uint64(seed), int(precision),
                            int(trial_steps), C.byref(t), C.byref(rate))
    if rc != TDS_OK:
        raise TdsError(rc, "autotune failed")
    return (dict(cells_per_particle=t.cells_per_particle, step_block=t.step_block, graph_steps=t.graph_steps,
                 lanes_per_particle=t.lanes_per_particle), rate.value)


def debug_seam_wrap(uv_old, uv, theta=None, vel=None, precision=64):
    """Device seam wrap on a batch of points (test hook)."""
    uo = np.ascontiguousarray(uv_old, np.float64)
    u = np.array(uv, np.float64, order="C")
    n = len(u)
    th = np.zeros(n) if theta is None else np.array(theta, np.float64)
    v = np.zeros((n, 2)) if vel is None else np.array(vel, np.float64, order="C")
    nw = np.zeros(n, np.int32)
    rc = lib().tds_debug_seam_wrap(n, uo.ctypes.data, u.ctypes.data, th.ctypes.data, v.ctypes.data, nw.ctypes.data,
                                   int(precision))
    if rc:
        raise TdsError(rc, "debug seam wrap failed")
    return u, th, v, nw
