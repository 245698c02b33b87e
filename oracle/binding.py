"""ctypes binding of the CPU oracle (test infrastructure only; see oracle/__init__.py).

Two builds of ``curvami_oracle.cpp`` land in ``oracle/_build/``:
  * ``liboracle.so``        -O2 -ffp-contract=off: the checker (fixed rounding, no FMA);
  * ``liboracle_native.so`` the reference's own release flags (CMakeLists.txt:124-143:
    -O2 and -march=native / -mcpu=native, OpenMP): the timed CPU baseline only.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "curvami_oracle.cpp")

_lock = threading.Lock()
_libs: dict[str, C.CDLL] = {}


def _native_flag() -> list[str]:
    m = platform.machine().lower()
    if m in ("aarch64", "arm64"):
        return ["-mcpu=native"]
    return ["-march=native"]


def build_oracle(force: bool = False) -> None:
    """Compile both oracle builds (seconds); skipped when up to date."""
    os.makedirs(BUILD, exist_ok=True)
    jobs = [
        ("liboracle.so", ["-O2", "-ffp-contract=off"]),
        ("liboracle_native.so", ["-O2"] + _native_flag()),
    ]
    procs = []
    for name, flags in jobs:
        out = os.path.join(BUILD, name)
        if (not force and os.path.exists(out)
                and os.path.getmtime(out) >= max(os.path.getmtime(SRC),
                                                 os.path.getmtime(SRC.replace(".cpp", ".h")))):
            continue
        cmd = ["g++", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-Wall"] + flags + [
            "-o", out + ".tmp", SRC]
        procs.append((subprocess.Popen(cmd), out))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed: {out}")
        os.replace(out + ".tmp", out)


class _Crease(C.Structure):
    _fields_ = [("xy", C.c_void_p), ("n_vertices", C.c_int), ("extend_start", C.c_int),
                ("extend_end", C.c_int), ("is_closed", C.c_int)]


class _Fold(C.Structure):
    _fields_ = [("n_gp", C.c_int),
                ("l_ptr", C.c_void_p), ("l_idx", C.c_void_p), ("l_dpsi", C.c_void_p),
                ("r_ptr", C.c_void_p), ("r_idx", C.c_void_p), ("r_dpsi", C.c_void_p),
                ("weight", C.c_void_p), ("tangent", C.c_void_p),
                ("Kt", C.c_double), ("theta0", C.c_double),
                ("theta0_gp", C.c_void_p), ("active", C.c_void_p)]


def load_oracle(native: bool = False) -> C.CDLL:
    name = "liboracle_native.so" if native else "liboracle.so"
    with _lock:
        if name in _libs:
            return _libs[name]
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build_oracle()
        lib = C.CDLL(path)
        vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
        lib.orc_frnn.restype = i64
        lib.orc_frnn.argtypes = [vp, i32, vp, i32, dbl, vp, vp, vp]
        lib.orc_frnn_var.restype = i64
        lib.orc_frnn_var.argtypes = [vp, i32, vp, vp, i32, vp, vp, vp]
        lib.orc_indicator.restype = None
        lib.orc_indicator.argtypes = [dbl, dbl, vp, vp]
        lib.orc_rkpm.restype = i32
        lib.orc_rkpm.argtypes = [vp, i32, vp, i32, vp, vp, vp, dbl, vp, i32, i32, vp, i32,
                                 vp, vp, vp, vp]
        lib.orc_abd_isotropic.restype = None
        lib.orc_abd_isotropic.argtypes = [dbl, dbl, dbl, vp, vp, vp]
        lib.orc_pattern.restype = i64
        lib.orc_pattern.argtypes = [i32, i32, vp, vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        lib.orc_pattern_new.restype = vp
        lib.orc_pattern_new.argtypes = [i32, i32, vp, vp, i32, vp, vp, vp, vp, C.POINTER(i64)]
        lib.orc_pattern_fill.restype = i64
        lib.orc_pattern_fill.argtypes = [vp, i32, i32, vp, vp, vp, vp, vp, vp, vp]
        lib.orc_pattern_free.restype = None
        lib.orc_pattern_free.argtypes = [vp]
        lib.orc_update_stiffness.restype = i32
        lib.orc_update_stiffness.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                             vp, i32, i32, vp, vp, vp]
        lib.orc_hinge.restype = i32
        lib.orc_hinge.argtypes = [i32, vp, i32, vp, i32, vp, vp, vp, vp, vp]
        lib.orc_fold_angle.restype = dbl
        lib.orc_fold_angle.argtypes = [vp, dbl, dbl, vp]
        lib.orc_hinge_energy.restype = dbl
        lib.orc_hinge_energy.argtypes = [vp, i32, vp]
        lib.orc_strain_energies.restype = None
        lib.orc_strain_energies.argtypes = [i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        lib.orc_kinematics.restype = None
        lib.orc_kinematics.argtypes = [i32, vp, vp, vp, vp, vp, vp, vp]
        lib.orc_set_static_schedule.restype = None
        lib.orc_set_static_schedule.argtypes = [i32]
        lib.orc_set_natural_curvature.restype = None
        lib.orc_set_natural_curvature.argtypes = [i32, dbl, dbl, dbl, dbl]
        _libs[name] = lib
        return lib


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Oracle:
    """Thin numpy front end over the oracle's C functions."""

    def __init__(self, native: bool = False):
        self.lib = load_oracle(native)

    # -- stage A ---------------------------------------------------------------------
    def frnn(self, node_xy, gp_xy, rho, rho_node=None):
        node_xy = _c(node_xy, np.float64)
        gp_xy = _c(gp_xy, np.float64)
        n_nodes, n_gp = len(node_xy), len(gp_xy)
        ptr = np.zeros(n_gp + 1, np.int64)
        if rho_node is None:
            nnz = self.lib.orc_frnn(_p(node_xy), n_nodes, _p(gp_xy), n_gp, float(rho), _p(ptr),
                                    None, None)
        else:
            rho_node = _c(rho_node, np.float64)
            nnz = self.lib.orc_frnn_var(_p(node_xy), n_nodes, _p(rho_node), _p(gp_xy), n_gp,
                                        _p(ptr), None, None)
        idx = np.zeros(max(nnz, 1), np.int32)
        s = np.zeros(max(nnz, 1), np.float64)
        if rho_node is None:
            self.lib.orc_frnn(_p(node_xy), n_nodes, _p(gp_xy), n_gp, float(rho), _p(ptr), _p(idx),
                              _p(s))
        else:
            self.lib.orc_frnn_var(_p(node_xy), n_nodes, _p(rho_node), _p(gp_xy), n_gp, _p(ptr),
                                  _p(idx), _p(s))
        return ptr, idx[:nnz], s[:nnz]

    @staticmethod
    def _creases(creases):
        keep = []
        arr = (_Crease * max(len(creases), 1))()
        for k, cr in enumerate(creases):
            xy = _c(cr["vertices"], np.float64).reshape(-1)
            keep.append(xy)
            arr[k].xy = xy.ctypes.data
            arr[k].n_vertices = len(xy) // 2
            arr[k].extend_start = int(cr.get("extend_start", False))
            arr[k].extend_end = int(cr.get("extend_end", False))
            arr[k].is_closed = int(cr.get("is_closed", False))
        return arr, keep

    def indicator(self, px, py, crease):
        arr, keep = self._creases([crease])
        out = np.zeros(8)
        self.lib.orc_indicator(float(px), float(py), C.addressof(arr), _p(out))
        del keep
        return out

    def rkpm(self, node_xy, gp_xy, ptr, idx, s, rho, order=2, creases=(), rho_node=None,
             kernel=0):
        node_xy = _c(node_xy, np.float64)
        gp_xy = _c(gp_xy, np.float64)
        ptr = _c(ptr, np.int64)
        idx = _c(idx, np.int32)
        s = _c(s, np.float64)
        nnz = int(ptr[-1])
        psi = np.zeros(max(nnz, 1))
        dpsi = np.zeros((max(nnz, 1), 2))
        ddpsi = np.zeros((max(nnz, 1), 3))
        bad = np.zeros(len(gp_xy), np.int8)
        arr, keep = self._creases(list(creases))
        rn = None if rho_node is None else _c(rho_node, np.float64)
        rc = self.lib.orc_rkpm(_p(node_xy), len(node_xy), _p(gp_xy), len(gp_xy), _p(ptr), _p(idx),
                               _p(s), float(rho), _p(rn), int(order), int(kernel),
                               C.addressof(arr), len(creases), _p(psi), _p(dpsi), _p(ddpsi),
                               _p(bad))
        del keep
        return psi[:nnz], dpsi[:nnz], ddpsi[:nnz], bad, rc

    # -- stage B ---------------------------------------------------------------------
    def abd(self, E, nu, h):
        A = np.zeros(9); B = np.zeros(9); D = np.zeros(9)
        self.lib.orc_abd_isotropic(float(E), float(nu), float(h), _p(A), _p(B), _p(D))
        return A.reshape(3, 3), B.reshape(3, 3), D.reshape(3, 3)

    def pattern(self, n_nodes, ptr, idx, folds=()):
        """Face (+ hinge union) pattern: outer, inner, col_ptr, col_nodes, map."""
        ptr = _c(ptr, np.int64)
        idx = _c(idx, np.int32)
        fl_ptr, fl_idx, fr_ptr, fr_idx, nf = _fold_lists(folds)
        outer = np.zeros(3 * n_nodes + 1, np.int32)
        n_gp = len(ptr) - 1
        nnz_c = C.c_int64(0)
        h = self.lib.orc_pattern_new(n_nodes, n_gp, _p(ptr), _p(idx), nf, _p(fl_ptr), _p(fl_idx),
                                     _p(fr_ptr), _p(fr_idx), C.byref(nnz_c))
        try:
            nnz = int(nnz_c.value)
            inner = np.zeros(max(nnz, 1), np.int32)
            col_ptr = np.zeros(n_nodes + 1, np.int64)
            nblk = nnz // 9
            col_nodes = np.zeros(max(nblk, 1), np.int32)
            n = np.diff(ptr)
            npairs = int((n * (n + 1) // 2).sum())
            mp = np.zeros(max(npairs, 1), np.int32)
            rc = self.lib.orc_pattern_fill(h, n_nodes, n_gp, _p(ptr), _p(idx), _p(outer), _p(inner), _p(col_ptr),
                                           _p(col_nodes), _p(mp))
        finally:
            self.lib.orc_pattern_free(h)
        if rc < 0:
            raise RuntimeError("Assembly: Gauss-point neighbour missing from the sparsity pattern; "
                               "CSR mapping is inconsistent.")
        return outer, inner[:nnz], col_ptr, col_nodes[:nblk], mp[:npairs]

    def set_natural_curvature(self, nc=None):
        """Kinematics::naturalCurvature() of the oracle (one field per process, as in the
        reference): nc = {"x0", "width", "angle_deg", "sense": "mountain" | "valley"} (the
        config's "natural_curvature" object, main.cpp:83-95), or None to switch it off.
        Assemblies, energies and kinematics given the points' coordinates (gp_xy) then use
        E1_el = E1 + kappa_bar(X)."""
        if nc is None:
            self.lib.orc_set_natural_curvature(0, 0.0, 1.0, 0.0, -1.0)
            return
        sign = -1.0 if nc.get("sense", "mountain") == "mountain" else 1.0
        self.lib.orc_set_natural_curvature(1, float(nc["x0"]), float(nc["width"]),
                                           float(nc["angle_deg"]) * np.pi / 180.0, sign)

    def update_stiffness(self, n_nodes, weight, ptr, idx, dpsi, ddpsi, outer, mp, x, A, B, D,
                         want_K=True, n_threads=1, gp_xy=None, static_schedule=False):
        """NonLinearAssembler::updateStiffness restated. static_schedule: a static split of
        the Gauss points over the threads instead of the reference's guided schedule, so
        that K and F are bitwise the same on every run with the same thread count."""
        weight = _c(weight, np.float64)
        ptr = _c(ptr, np.int64)
        idx = _c(idx, np.int32)
        dpsi = _c(dpsi, np.float64)
        ddpsi = _c(ddpsi, np.float64)
        x = _c(x, np.float64)
        A = _c(A, np.float64); B = _c(B, np.float64); D = _c(D, np.float64)
        nnz = int(outer[-1])
        K = np.zeros(max(nnz, 1)) if want_K else None
        F = np.zeros(3 * n_nodes)
        self.lib.orc_set_static_schedule(int(bool(static_schedule)))
        self.lib.orc_update_stiffness(n_nodes, len(ptr) - 1, _p(weight), _p(ptr), _p(idx),
                                      _p(dpsi), _p(ddpsi), _p(_c(outer, np.int32)),
                                      _p(_c(mp, np.int32)), _p(x), _p(A), _p(B), _p(D),
                                      int(want_K), int(n_threads), _p(K), _p(F),
                                      _p(None if gp_xy is None else _c(gp_xy, np.float64)))
        return (K[:nnz] if want_K else None), F

    def hinge(self, n_nodes, x, folds, outer=None, col_ptr=None, col_nodes=None, K=None, F=None,
              exact_tangent=False):
        x = _c(x, np.float64)
        arr, keep = _fold_structs(folds)
        if F is None:
            F = np.zeros(3 * n_nodes)
        rc = self.lib.orc_hinge(n_nodes, _p(x), len(folds), C.addressof(arr), int(exact_tangent),
                                _p(None if outer is None else _c(outer, np.int32)),
                                _p(None if col_ptr is None else _c(col_ptr, np.int64)),
                                _p(None if col_nodes is None else _c(col_nodes, np.int32)),
                                _p(K), _p(F))
        del keep
        if rc != 0:
            raise RuntimeError("hinge block outside the union pattern")
        return K, F

    def fold_angle(self, F12, tx, ty, want_grad=True):
        F12 = _c(F12, np.float64)
        g = np.zeros(12) if want_grad else None
        th = self.lib.orc_fold_angle(_p(F12), float(tx), float(ty), _p(g))
        return th, g

    def hinge_energy(self, x, folds):
        arr, keep = _fold_structs(folds)
        e = self.lib.orc_hinge_energy(_p(_c(x, np.float64)), len(folds), C.addressof(arr))
        del keep
        return e

    def strain_energies(self, weight, ptr, idx, dpsi, ddpsi, x, A, B, D, gp_xy=None):
        em = C.c_double(); eb = C.c_double()
        self.lib.orc_strain_energies(len(ptr) - 1, _p(_c(weight, np.float64)), _p(_c(ptr, np.int64)),
                                     _p(_c(idx, np.int32)), _p(_c(dpsi, np.float64)),
                                     _p(_c(ddpsi, np.float64)), _p(_c(x, np.float64)),
                                     _p(_c(A, np.float64)), _p(_c(B, np.float64)),
                                     _p(_c(D, np.float64)), C.byref(em), C.byref(eb),
                                     _p(None if gp_xy is None else _c(gp_xy, np.float64)))
        return em.value, eb.value

    def kinematics(self, g, ptr, idx, dpsi, ddpsi, x, X=None):
        """Kinematics::compute at point g: r0X r0Y r0XX r0YY r0XY b (3 each), C0^-1 (4), E0
        (xx yy xy), E1 (xx yy xy), E1_el (xx yy xy; X = the point's reference coordinates)."""
        out = np.zeros(31)
        self.lib.orc_kinematics(int(g), _p(_c(ptr, np.int64)), _p(_c(idx, np.int32)),
                                _p(_c(dpsi, np.float64)), _p(_c(ddpsi, np.float64)),
                                _p(_c(x, np.float64)), _p(out), _p(None if X is None else _c(X, np.float64)))
        return out


def _fold_lists(folds):
    """Concatenate every fold's left/right neighbour lists (pattern input)."""
    if not folds:
        return None, None, None, None, 0
    lp, li, rp, ri = [np.zeros(1, np.int64)], [], [np.zeros(1, np.int64)], []
    loff = roff = 0
    n = 0
    for f in folds:
        lptr = np.asarray(f["left"]["ptr"], np.int64)
        rptr = np.asarray(f["right"]["ptr"], np.int64)
        lp.append(lptr[1:] + loff); rp.append(rptr[1:] + roff)
        li.append(np.asarray(f["left"]["idx"], np.int32)); ri.append(np.asarray(f["right"]["idx"], np.int32))
        loff += int(lptr[-1]); roff += int(rptr[-1])
        n += len(lptr) - 1
    return (np.concatenate(lp), np.concatenate(li) if li else np.zeros(1, np.int32),
            np.concatenate(rp), np.concatenate(ri) if ri else np.zeros(1, np.int32), n)


def _fold_structs(folds):
    arr = (_Fold * max(len(folds), 1))()
    keep = []
    for k, f in enumerate(folds):
        L, R = f["left"], f["right"]
        items = {
            "l_ptr": _c(L["ptr"], np.int64), "l_idx": _c(L["idx"], np.int32),
            "l_dpsi": _c(L["dpsi"], np.float64), "r_ptr": _c(R["ptr"], np.int64),
            "r_idx": _c(R["idx"], np.int32), "r_dpsi": _c(R["dpsi"], np.float64),
            "weight": _c(f["weight"], np.float64), "tangent": _c(f["tangent"], np.float64),
        }
        keep.append(items)
        arr[k].n_gp = len(items["l_ptr"]) - 1
        for name, a in items.items():
            setattr(arr[k], name, a.ctypes.data)
        arr[k].Kt = float(f["Kt"])
        arr[k].theta0 = float(f.get("theta0", 0.0))
        t0 = f.get("theta0_gp")
        act = f.get("active")
        if t0 is not None:
            t0 = _c(t0, np.float64); keep.append(t0); arr[k].theta0_gp = t0.ctypes.data
        if act is not None:
            act = _c(act, np.int8); keep.append(act); arr[k].active = act.ctypes.data
    return arr, keep
