"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes bindings over oracle/_build/liboracle.so (the FP64 CPU restatement of 2DTissue's
per-step update, see oracle.h). Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm import this package, and only as the checker.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u32 = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_philox4x32_10.argtypes = [_u32, _u32, _u32]
        L.orc_ref_angles_to_unit_vectors.argtypes = [_i, C.c_int, _d]
        L.orc_ref_repulsive_adhesion.argtypes = [C.c_double] * 7 + [_d]
        L.orc_ref_mean_angle_deg.argtypes = [_d, C.c_int, C.POINTER(C.c_double)]
        L.orc_ref_symmetrize_min.argtypes = [_d, C.c_int]
        L.orc_ref_dist_vect.argtypes = [_d, C.c_int, _d, _d]
        L.orc_ref_average_n.argtypes = [_d, _i, C.c_int, C.c_double, _i]
        L.orc_ref_seam_wrap.argtypes = [_d, _d, _i, C.c_int]
        L.orc_ref_step.argtypes = [C.c_int, _d, C.c_int, _i, C.c_int, _d, _i, _i, _d] + [C.c_double] * 6 + [
            C.c_int, _d, _i, _i, _d, _d, _i, _d]
        L.orc_mesh_create.restype = C.c_void_p
        L.orc_mesh_create.argtypes = [C.c_int, _d, C.c_int, _i, C.c_int, _d, _i]
        L.orc_mesh_free.argtypes = [C.c_void_p]
        L.orc_mesh_face_data.argtypes = [C.c_void_p, C.c_int, _d, _d, _d]
        L.orc_mesh_locate.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int)]
        L.orc_mesh_map.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, _d]
        L.orc_model_wrap.argtypes = [_d, _d, _d, _d, C.c_int, C.POINTER(C.c_int)]
        L.orc_model_step.argtypes = [C.c_void_p, _d, C.c_int, C.c_uint64, C.c_int64, C.c_int, _d, C.c_int,
                                     _d, _d, _i, _d, _i, C.c_void_p, C.c_int, C.c_void_p,
                                     _d, _d, _i, _d, _d, _i, _i, _d, C.POINTER(C.c_int), C.c_int]
        L.orc_model_step_dual.argtypes = [C.c_void_p, _d, _d, C.c_int, C.c_uint64, C.c_int64, C.c_int, _d,
                                          C.c_int, _d, _d, _d, _d, _i, _d, _d, _i, C.c_void_p,
                                          _d, _d, _d, _d, _i, _d, _d, _d, _d]
        _lib = L
    return _lib


def philox4x32_10(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def ref_angles_to_unit_vectors(deg):
    deg = np.ascontiguousarray(deg, np.int32)
    out = np.zeros((len(deg), 2))
    lib().orc_ref_angles_to_unit_vectors(deg, len(deg), out)
    return out


def ref_repulsive_adhesion(k, sigma, dist, r_adh, k_adh, dist_v):
    out = np.zeros(2)
    lib().orc_ref_repulsive_adhesion(k, sigma, dist, r_adh, k_adh, float(dist_v[0]), float(dist_v[1]), out)
    return out


def ref_mean_angle_deg(angles):
    a = np.ascontiguousarray(angles, np.float64)
    out = C.c_double()
    rc = lib().orc_ref_mean_angle_deg(a, len(a), C.byref(out))
    if rc != 0:
        raise ValueError("The input vector should not be empty.")
    return out.value


def ref_symmetrize_min(A):
    A = np.array(A, np.float64, order="C")
    lib().orc_ref_symmetrize_min(A, A.shape[0])
    return A


def ref_dist_vect(r):
    r = np.ascontiguousarray(r, np.float64)
    n = r.shape[0]
    dx, dy = np.zeros((n, n)), np.zeros((n, n))
    lib().orc_ref_dist_vect(r, n, dx, dy)
    return dx, dy


def ref_average_n(dist_length, n, sigma):
    dl = np.ascontiguousarray(dist_length, np.float64)
    n = np.ascontiguousarray(n, np.int32)
    out = np.zeros_like(n)
    if lib().orc_ref_average_n(dl, n, len(n), sigma, out) != 0:
        raise ValueError("empty neighbourhood")
    return out


def ref_seam_wrap(uv_old, uv, n_deg):
    uo = np.array(uv_old, np.float64, order="C")
    u = np.array(uv, np.float64, order="C")
    n = np.array(n_deg, np.int32)
    if lib().orc_ref_seam_wrap(uo, u, n, len(n)) != 0:
        raise RuntimeError("ref seam wrap did not terminate")
    return u, n, uo


def ref_step(arrays, dist_vv, params, r_uv, n_deg, nearest):
    """One ref-form step (orc_ref_step) from (r_uv, n_deg, nearest); params holds the _2DTissue
    ctor values v0, k, sigma, r_adh, k_adh, step_size. Returns the new state and the step's order
    parameter."""
    v3 = np.ascontiguousarray(arrays["v3"], np.float64)
    f3 = np.ascontiguousarray(arrays["f3"], np.int32)
    uv = np.ascontiguousarray(arrays["uv"], np.float64)
    fuv = np.ascontiguousarray(arrays["fuv"], np.int32)
    uv2v = np.ascontiguousarray(arrays["uv2v"], np.int32)
    D = np.ascontiguousarray(dist_vv, np.float64)
    u = np.array(r_uv, np.float64, order="C")
    n = np.array(n_deg, np.int32)
    near = np.array(nearest, np.int32)
    N = len(n)
    r3d, rdot, nbr, order = np.zeros((N, 3)), np.zeros((N, 2)), np.zeros(N, np.int32), np.zeros(1)
    rc = lib().orc_ref_step(len(v3), v3, len(f3), f3, len(uv), uv, fuv, uv2v, D, params["v0"], params["k"],
                            params["sigma"], params["r_adh"], params["k_adh"], params["step_size"], N, u, n, near,
                            r3d, rdot, nbr, order)
    if rc != 0:
        raise RuntimeError("orc_ref_step failed (%d)" % rc)
    return dict(uv=u, n_deg=n, nearest=near, r3d=r3d, r_dot=rdot, nbr=nbr, order=float(order[0]))


def model_wrap(s_uv, e_uv, theta, vuv, max_wraps=8):
    s = np.array(s_uv, np.float64)
    e = np.array(e_uv, np.float64)
    th = np.array([theta], np.float64)
    v = np.array(vuv, np.float64)
    nw = C.c_int()
    rc = lib().orc_model_wrap(s, e, th, v, max_wraps, C.byref(nw))
    return e, float(th[0]), v, nw.value, rc


class Mesh:
    """Oracle-side mesh: per-face chart maps and its own UV bin grid (built from raw arrays)."""

    def __init__(self, v3, f3, uv, fuv):
        self.v3 = np.ascontiguousarray(v3, np.float64).reshape(-1, 3)
        self.f3 = np.ascontiguousarray(f3, np.int32).reshape(-1, 3)
        self.uv = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
        self.fuv = np.ascontiguousarray(fuv, np.int32).reshape(-1, 3)
        self.h = lib().orc_mesh_create(len(self.v3), self.v3.ravel(), len(self.f3), self.f3.ravel(),
                                       len(self.uv), self.uv.ravel(), self.fuv.ravel())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mesh_free(self.h)
            self.h = None

    @property
    def F(self):
        return len(self.f3)

    def face_data(self, f):
        J, Jp, n = np.zeros(6), np.zeros(6), np.zeros(3)
        lib().orc_mesh_face_data(self.h, int(f), J, Jp, n)
        return J, Jp, n

    def locate(self, u, v, f_old=-1):
        mode = C.c_int()
        f = lib().orc_mesh_locate(self.h, float(u), float(v), int(f_old), C.byref(mode))
        return f, mode.value

    def map(self, f, u, v):
        r = np.zeros(3)
        lib().orc_mesh_map(self.h, int(f), float(u), float(v), r)
        return r


PARAM_ORDER = ("R", "k", "k_adh", "r_max", "v0", "mu", "tau", "align", "eta", "dt")


def params_array(p):
    return np.array([float(p[k]) for k in PARAM_ORDER], np.float64)


def model_step(mesh, params, state, step, seed, local_bits=31, centroid=(0.0, 0.0, 0.0), noise=None, subset=None,
               force_mode=0, threads=0):
    """One model-form step. `state` has uv (N,2), theta (N,), face (N,), r3d (N,3), ids (N,).
    Returns a dict of outputs for `subset` (or all particles) plus phi_sums and status."""
    uv = np.ascontiguousarray(state["uv"], np.float64).reshape(-1, 2)
    N = uv.shape[0]
    th = np.ascontiguousarray(state["theta"], np.float64)
    fc = np.ascontiguousarray(state["face"], np.int32)
    r3 = np.ascontiguousarray(state["r3d"], np.float64).reshape(-1, 3)
    ids = np.ascontiguousarray(state.get("ids", np.arange(N)), np.int32)
    nz = None if noise is None else np.ascontiguousarray(noise, np.float64)
    sub = None if subset is None else np.ascontiguousarray(subset, np.int32)
    n = N if sub is None else len(sub)
    out = dict(uv=np.zeros((n, 2)), theta=np.zeros(n), face=np.zeros(n, np.int32), r3d=np.zeros((n, 3)),
               vel_uv=np.zeros((n, 2)), nbr=np.zeros(n, np.int32), wraps=np.zeros(n, np.int32),
               phi_sums=np.zeros(6))
    st = C.c_int()
    lib().orc_model_step(mesh.h, params_array(params), int(force_mode), C.c_uint64(seed), C.c_int64(step),
                         int(local_bits), np.ascontiguousarray(centroid, np.float64), N, uv.ravel(), th, fc,
                         r3.ravel(), ids, None if nz is None else nz.ctypes.data, n,
                         None if sub is None else sub.ctypes.data, out["uv"].ravel(), out["theta"], out["face"],
                         out["r3d"].ravel(), out["vel_uv"].ravel(), out["nbr"], out["wraps"], out["phi_sums"],
                         C.byref(st), int(threads))
    out["status"] = st.value
    return out


def model_step_dual(mesh, params, dparams, state, dstate, step, seed, local_bits=31, centroid=(0.0, 0.0, 0.0),
                    noise=None, force_mode=0):
    """Forward-mode tangent of one model-form step over all particles."""
    uv = np.ascontiguousarray(state["uv"], np.float64).reshape(-1, 2)
    N = uv.shape[0]
    th = np.ascontiguousarray(state["theta"], np.float64)
    fc = np.ascontiguousarray(state["face"], np.int32)
    r3 = np.ascontiguousarray(state["r3d"], np.float64).reshape(-1, 3)
    ids = np.ascontiguousarray(state.get("ids", np.arange(N)), np.int32)
    duv = np.ascontiguousarray(dstate["uv"], np.float64).reshape(-1, 2)
    dth = np.ascontiguousarray(dstate["theta"], np.float64)
    dr3 = np.ascontiguousarray(dstate["r3d"], np.float64).reshape(-1, 3)
    nz = None if noise is None else np.ascontiguousarray(noise, np.float64)
    out = dict(uv=np.zeros((N, 2)), duv=np.zeros((N, 2)), theta=np.zeros(N), dtheta=np.zeros(N),
               face=np.zeros(N, np.int32), r3d=np.zeros((N, 3)), dr3d=np.zeros((N, 3)), phi_sums=np.zeros(6),
               dphi_sums=np.zeros(6))
    rc = lib().orc_model_step_dual(mesh.h, params_array(params), params_array(dparams), int(force_mode),
                                   C.c_uint64(seed), C.c_int64(step), int(local_bits),
                                   np.ascontiguousarray(centroid, np.float64), N, uv.ravel(), duv.ravel(), th, dth,
                                   fc, r3.ravel(), dr3.ravel(), ids, None if nz is None else nz.ctypes.data,
                                   out["uv"].ravel(), out["duv"].ravel(), out["theta"], out["dtheta"],
                                   out["face"], out["r3d"].ravel(), out["dr3d"].ravel(), out["phi_sums"],
                                   out["dphi_sums"])
    out["status"] = rc
    return out
