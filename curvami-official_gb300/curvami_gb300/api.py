"""Host-side mirror of the reference's hot-path interface over the C ABI.

Names follow the reference's call sites:
  * ``shape_functions`` = GlobalFRNN::execute + GlobalRKPM::solve for one domain
    (core/include/curvami/FRNN.h:23, GlobalRKPM.h:19), as SetupHelper::
    recomputeShapeFunctions calls them (plate/SetupHelper.h:112-138);
  * ``NonLinearAssembler`` = the assembler (plate/Assembly.h:18-346) with the hinge of
    Meshless::assembleSystem (plate/Meshless.h:102-127);
  * ``Meshless``-style helpers ``assemble_system`` / ``assemble_internal_only``.
Errors raise CGBError carrying the reference's message where it has one.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Context:
    """One GPU, one stream (cgb_context)."""

    def __init__(self, device: int = 0):
        self.lib = L.load_library()
        h = C.c_void_p()
        rc = self.lib.cgb_create(device, C.byref(h))
        if rc != L.CGB_OK:
            raise L.CGBError(rc, f"cgb_create failed (status {rc}): no usable CUDA device")
        self.h = h
        self._keep = []
        self.natural_curvature = None

    def check(self, rc: int):
        if rc != L.CGB_OK:
            msg = self.lib.cgb_last_error(self.h).decode(errors="replace")
            raise L.CGBError(rc, msg)

    def set_nodes(self, node_xy):
        self.node_xy = _c(node_xy, np.float64)
        self.n_nodes = len(self.node_xy)
        self.check(self.lib.cgb_set_nodes(self.h, _p(self.node_xy), self.n_nodes))

    def synchronize(self):
        self.check(self.lib.cgb_synchronize(self.h))

    def set_natural_curvature(self, nc=None):
        """Kinematics::naturalCurvature() for every constitutive evaluation of this context
        (cgb_set_natural_curvature): nc is the config's "natural_curvature" object
        (main.cpp:83-95: {"x0", "width", "angle_deg", "sense": "mountain" | "valley"}), or
        None to switch it off."""
        v = L.NaturalCurvature()
        if nc is not None:
            sense = nc.get("sense", "mountain")
            if sense not in ("mountain", "valley"):
                raise ValueError("natural_curvature.sense must be mountain or valley")
            v.active = 1
            v.x0, v.width = float(nc["x0"]), float(nc["width"])
            v.theta0 = float(nc["angle_deg"]) * np.pi / 180.0
            v.sign = -1.0 if sense == "mountain" else 1.0
        self.check(self.lib.cgb_set_natural_curvature(self.h, C.byref(v)))
        self.natural_curvature = None if nc is None else dict(nc)

    def set_stream(self, stream_ptr: int):
        """Launch on the caller's cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self.check(self.lib.cgb_set_stream(self.h, C.c_void_p(stream_ptr)))

    def profile(self, on: bool):
        self.check(self.lib.cgb_profile_enable(self.h, int(bool(on))))

    def profile_read(self, reset: bool = True):
        """Per-phase device ms and kernel launches since the last reset."""
        ms = np.zeros(len(L.PHASES))
        n = np.zeros(len(L.PHASES), np.int64)
        self.check(self.lib.cgb_profile_read(self.h, _p(ms), _p(n), int(bool(reset))))
        return dict(zip(L.PHASES, ms)), dict(zip(L.PHASES, n))

    def close(self):
        if getattr(self, "h", None):
            self.lib.cgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _creases_struct(creases):
    arr = (L.Crease * max(len(creases), 1))()
    keep = []
    for k, cr in enumerate(creases):
        xy = _c(cr["vertices"], np.float64).reshape(-1)
        keep.append(xy)
        arr[k].xy = xy.ctypes.data
        arr[k].n_vertices = len(xy) // 2
        arr[k].extend_start = int(bool(cr.get("extend_start", False)))
        arr[k].extend_end = int(bool(cr.get("extend_end", False)))
        arr[k].is_closed = int(bool(cr.get("is_closed", False)))
    return arr, keep


class ShapeSet:
    """Device-resident neighbour lists and shape functions of one point set (cgb_shape)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.h = handle
        n = C.c_int(); nnz = C.c_int64(); mx = C.c_int()
        ctx.check(ctx.lib.cgb_shape_size(self.h, C.byref(n), C.byref(nnz), C.byref(mx)))
        self.n_gp, self.nnz, self.max_n = n.value, nnz.value, mx.value

    def rebuild(self, creases=()):
        """cgb_shape_rebuild: Phi and its derivatives recomputed in place for other cuts
        (SetupHelper::recomputeShapeFunctions, plate/SetupHelper.h:112-138); the points and
        neighbour lists stay. Raises CGBError with the reference's message on a
        rank-deficient support (the new, flagged values then stand)."""
        arr, keep = _creases_struct(list(creases))
        rc = self.ctx.lib.cgb_shape_rebuild(self.h, C.addressof(arr), len(creases))
        del keep
        self.ctx.check(rc)

    def download(self):
        ptr = np.zeros(self.n_gp + 1, np.int64)
        idx = np.zeros(max(self.nnz, 1), np.int32)
        s = np.zeros(max(self.nnz, 1))
        psi = np.zeros(max(self.nnz, 1))
        dpsi = np.zeros((max(self.nnz, 1), 2))
        ddpsi = np.zeros((max(self.nnz, 1), 3))
        self.ctx.check(self.ctx.lib.cgb_shape_download(self.h, _p(ptr), _p(idx), _p(s), _p(psi), _p(dpsi),
                                                        _p(ddpsi)))
        k = self.nnz
        return {"ptr": ptr, "idx": idx[:k], "s": s[:k], "psi": psi[:k], "dpsi": dpsi[:k],
                "ddpsi": ddpsi[:k]}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.cgb_shape_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def concat_shapes(ctx: Context, sets, node_offsets) -> ShapeSet:
    """cgb_shape_concat: the union of several shape sets, set k's neighbour indices shifted
    by node_offsets[k] (independent plates stacked over the union of their nodes)."""
    arr = (C.c_void_p * len(sets))(*[st.h for st in sets])
    off = _c(node_offsets, np.int32)
    h = C.c_void_p()
    ctx.check(ctx.lib.cgb_shape_concat(ctx.h, arr, _p(off), len(sets), C.byref(h)))
    return ShapeSet(ctx, h)


SHAPE_PRECISIONS = {"fp64": 0, "mixed": 1}


def shape_functions(ctx: Context, gp_xy, rho, order=2, creases=(), rho_node=None, kernel=0,
                    precision="fp64") -> ShapeSet:
    """GlobalFRNN::execute + GlobalRKPM::solve for one set of Gauss points. Raises
    CGBError (CGB_ERR_SINGULAR / CGB_ERR_PIVOT) with the reference's message on a
    rank-deficient support. precision "fp64" is the reference's arithmetic; "mixed" sums
    the per-neighbour terms in FP32 pairs and factors the moment matrix in FP64."""
    gp_xy = _c(gp_xy, np.float64)
    prm = L.ShapeParams()
    prm.rho = float(rho)
    rn = None if rho_node is None else _c(rho_node, np.float64)
    prm.rho_node = _p(rn)
    prm.order = int(order)
    prm.kernel = int(kernel)
    if precision not in SHAPE_PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(SHAPE_PRECISIONS)}")
    prm.precision = SHAPE_PRECISIONS[precision]
    arr, keep = _creases_struct(list(creases))
    h = C.c_void_p()
    rc = ctx.lib.cgb_shape_build(ctx.h, _p(gp_xy), len(gp_xy), C.byref(prm), C.addressof(arr),
                                 len(creases), C.byref(h))
    del keep
    if rc != L.CGB_OK:
        msg = ctx.lib.cgb_last_error(ctx.h).decode(errors="replace")
        if h.value:
            ctx.lib.cgb_shape_destroy(h)
        raise L.CGBError(rc, msg)
    return ShapeSet(ctx, h)


def shape_from_host(ctx: Context, ptr, idx, dpsi, ddpsi, psi=None) -> ShapeSet:
    ptr = _c(ptr, np.int64); idx = _c(idx, np.int32)
    dpsi = _c(dpsi, np.float64); ddpsi = _c(ddpsi, np.float64)
    psi = None if psi is None else _c(psi, np.float64)
    h = C.c_void_p()
    ctx.check(ctx.lib.cgb_shape_from_host(ctx.h, len(ptr) - 1, _p(ptr), _p(idx), _p(psi), _p(dpsi),
                                          _p(ddpsi), C.byref(h)))
    return ShapeSet(ctx, h)


class NonLinearAssembler:
    """initSparsityPattern at construction (face + hinge union), then assemble()."""

    def __init__(self, ctx: Context, faces: ShapeSet, face_weight, folds=()):
        self.ctx = ctx
        self.faces = faces
        self.face_weight = _c(face_weight, np.float64)
        arr = (L.Fold * max(len(folds), 1))()
        keep = []
        for k, f in enumerate(folds):
            w = _c(f["weight"], np.float64); t = _c(f["tangent"], np.float64)
            keep += [w, t]
            arr[k].left = f["left"].h
            arr[k].right = f["right"].h
            arr[k].weight = w.ctypes.data
            arr[k].tangent = t.ctypes.data
            arr[k].Kt = float(f["Kt"])
            arr[k].theta0 = float(f.get("theta0", 0.0))
            if f.get("theta0_gp") is not None:
                t0 = _c(f["theta0_gp"], np.float64); keep.append(t0); arr[k].theta0_gp = t0.ctypes.data
            if f.get("active") is not None:
                ac = _c(f["active"], np.int8); keep.append(ac); arr[k].active = ac.ctypes.data
        self.folds = list(folds)
        h = C.c_void_p()
        ctx.check(ctx.lib.cgb_assembler_create(ctx.h, faces.h, _p(self.face_weight), C.addressof(arr),
                                               len(folds), C.byref(h)))
        del keep
        self.h = h
        nd = C.c_int(); nnz = C.c_int64()
        ctx.check(ctx.lib.cgb_assembler_pattern(self.h, C.byref(nd), C.byref(nnz)))
        self.n_dofs, self.nnz = nd.value, nnz.value

    def set_fold_state(self, fold: int, theta0: float = 0.0, theta0_gp=None, active=None):
        """cgb_assembler_set_fold_state: Fold::gp_theta0 / gp_active of one fold (None = the
        scalar rest angle everywhere / every point active)."""
        t0 = None if theta0_gp is None else _c(theta0_gp, np.float64)
        ac = None if active is None else _c(np.asarray(active) != 0, np.int8)
        self.ctx.check(self.ctx.lib.cgb_assembler_set_fold_state(self.h, int(fold), float(theta0), _p(t0),
                                                                  _p(ac)))

    def set_material(self, A, B, D):
        self.A, self.B, self.D = (_c(A, np.float64).reshape(9), _c(B, np.float64).reshape(9),
                                  _c(D, np.float64).reshape(9))
        self.ctx.check(self.ctx.lib.cgb_set_material(self.h, _p(self.A), _p(self.B), _p(self.D)))

    def pattern(self):
        outer = np.zeros(self.n_dofs + 1, np.int32)
        inner = np.zeros(max(self.nnz, 1), np.int32)
        self.ctx.check(self.ctx.lib.cgb_assembler_download_pattern(self.h, _p(outer), _p(inner)))
        return outer, inner[: self.nnz]

    def stats(self):
        """{"pairs", "blocks", "entries", "direct_groups"}: sizes of the assembler's work."""
        out = np.zeros(4, np.int64)
        self.ctx.check(self.ctx.lib.cgb_assembler_stats(self.h, _p(out)))
        return dict(zip(("pairs", "blocks", "entries", "direct_groups"), (int(v) for v in out)))

    def tensor_stats(self):
        """{"tensor_groups", "core_groups", "point_cols", "ctas_per_sm"}: the tensor-core
        tangent's share (groups of 16 points as one tensor-core product, groups left to the
        CUDA cores, the sum of points x MMA columns, i.e. 10,240 x point_cols TF32 flops per
        assembly) and the CTAs per SM of its last launch."""
        out = np.zeros(4, np.int64)
        self.ctx.check(self.ctx.lib.cgb_assembler_tensor_stats(self.h, _p(out)))
        return dict(zip(("tensor_groups", "core_groups", "point_cols", "ctas_per_sm"), (int(v) for v in out)))

    def csr_mapping(self):
        n = np.diff(self.faces.download()["ptr"])
        total = int((n * (n + 1) // 2).sum())
        m = np.zeros(max(total, 1), np.int32)
        self.ctx.check(self.ctx.lib.cgb_assembler_download_map(self.h, _p(m), total))
        return m[:total]

    def assemble(self, x, flags=L.TANGENT | L.HINGE, K_out=None, F_out=None):
        """Host buffers in and out (cgb_assemble)."""
        x = _c(x, np.float64)
        F = F_out if F_out is not None else np.empty(self.n_dofs)
        K = None
        if flags & L.TANGENT:
            K = K_out if K_out is not None else np.empty(max(self.nnz, 1))
        self.ctx.check(self.ctx.lib.cgb_assemble(self.h, _p(x), _p(K), _p(F), int(flags)))
        return (K[: self.nnz] if K is not None else None), F

    def assemble_device(self, d_x: int, d_K: int | None, d_F: int, flags):
        """Device pointers (cgb_assemble_device), asynchronous on the context stream."""
        self.ctx.check(self.ctx.lib.cgb_assemble_device(self.h, C.c_void_p(d_x),
                                                        C.c_void_p(d_K) if d_K else None,
                                                        C.c_void_p(d_F), int(flags)))

    def set_tuning(self, n_chunks=0, residual_threads=0, tangent_ctas_per_sm=0, tangent_kind=0):
        """cgb_assembler_set_tuning (0 = the library's default; tangent_kind 0 the CUDA-core
        tangent, 1 the tensor-core one)."""
        t = L.Tuning(int(n_chunks), int(residual_threads), int(tangent_ctas_per_sm), int(tangent_kind))
        self.ctx.check(self.ctx.lib.cgb_assembler_set_tuning(self.h, C.byref(t)))
        self.tuning = (int(n_chunks), int(residual_threads), int(tangent_ctas_per_sm), int(tangent_kind))

    def graph(self, d_x: int, d_K: int | None, d_F: int, flags) -> "AssemblyGraph":
        """One cgb_assemble_device call on these device buffers captured as a CUDA graph."""
        return AssemblyGraph(self, d_x, d_K, d_F, flags)

    def energies(self, x):
        x = _c(x, np.float64)
        em = C.c_double(); eb = C.c_double(); eh = C.c_double()
        self.ctx.check(self.ctx.lib.cgb_energies(self.h, _p(x), C.byref(em), C.byref(eb), C.byref(eh)))
        return em.value, eb.value, eh.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.cgb_assembler_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AssemblyGraph:
    """cgb_graph: replay of one captured assembly with a single graph launch."""

    def __init__(self, asm: NonLinearAssembler, d_x, d_K, d_F, flags):
        self.asm = asm
        self.ctx = asm.ctx
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.cgb_graph_create(asm.h, C.c_void_p(d_x), C.c_void_p(d_K) if d_K else None,
                                                     C.c_void_p(d_F), int(flags), C.byref(h)))
        self.h = h

    def launch(self):
        self.ctx.check(self.ctx.lib.cgb_graph_launch(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.cgb_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def abd_isotropic(E: float, nu: float, h: float):
    """A, B, D of one isotropic ply (main.cpp:53-61 through Constitutive::computeABD,
    plate/Constitutive.h:10-50): Q = E/(1-nu^2) [[1, nu, 0], [nu, 1, 0], [0, 0, (1-nu)/2]]."""
    den = 1.0 - nu * nu
    G = E / (2.0 * (1.0 + nu))
    Q = np.array([[E / den, nu * E / den, 0.0], [nu * E / den, E / den, 0.0], [0.0, 0.0, G]])
    z0, z1 = -h / 2.0, h / 2.0
    return Q * (z1 - z0), 0.5 * Q * (z1 * z1 - z0 * z0), (1.0 / 3.0) * Q * (z1 ** 3 - z0 ** 3)


def abd_laminate(plies):
    """A, B, D of a laminate by classical lamination theory (Constitutive::computeABD,
    plate/Constitutive.h:10-50): plies = [(E1, E2, nu12, G12, angle_deg, thickness), ...]
    from the bottom face up, the mid-plane at half the total thickness. Each ply's reduced
    stiffness Q is rotated to Q-bar by the ply angle and integrated through its thickness
    (A: 1, B: z, D: z^2). An unsymmetric layup gives B != 0 (membrane-bending coupling)."""
    h = float(sum(p[5] for p in plies))
    z = -h / 2.0
    A = np.zeros((3, 3)); B = np.zeros((3, 3)); D = np.zeros((3, 3))
    for E1, E2, nu12, G12, angle, t in plies:
        nu21 = (E2 / E1) * nu12
        den = 1.0 - nu12 * nu21
        Q11, Q22, Q12, Q66 = E1 / den, E2 / den, nu12 * E2 / den, G12
        th = np.deg2rad(angle)
        m, n = np.cos(th), np.sin(th)
        m2, n2 = m * m, n * n
        Qb = np.empty((3, 3))
        Qb[0, 0] = Q11 * m2 * m2 + 2.0 * (Q12 + 2.0 * Q66) * m2 * n2 + Q22 * n2 * n2
        Qb[1, 1] = Q11 * n2 * n2 + 2.0 * (Q12 + 2.0 * Q66) * m2 * n2 + Q22 * m2 * m2
        Qb[0, 1] = Qb[1, 0] = (Q11 + Q22 - 4.0 * Q66) * m2 * n2 + Q12 * (m2 * m2 + n2 * n2)
        Qb[0, 2] = Qb[2, 0] = (Q11 - Q12 - 2.0 * Q66) * n * m * m2 + (Q12 - Q22 + 2.0 * Q66) * n2 * n * m
        Qb[1, 2] = Qb[2, 1] = (Q11 - Q12 - 2.0 * Q66) * m * n * n2 + (Q12 - Q22 + 2.0 * Q66) * m2 * m * n
        Qb[2, 2] = (Q11 + Q22 - 2.0 * Q12 - 2.0 * Q66) * m2 * n2 + Q66 * (m2 * m2 + n2 * n2)
        z1 = z + t
        A += Qb * (z1 - z)
        B += 0.5 * Qb * (z1 * z1 - z * z)
        D += (1.0 / 3.0) * Qb * (z1 ** 3 - z ** 3)
        z = z1
    return A, B, D


class PlateModel:
    """A synthetic plate (synth.Plate) on the GPU: shape functions of the faces and of
    every fold side, the assembler with the hinge union pattern and the material."""

    def __init__(self, plate, ctx: Context | None = None, shape_precision: str = "fp64"):
        self.plate = plate
        self.ctx = ctx or Context(0)
        self.ctx.set_nodes(plate.node_xy)
        kw = dict(rho=plate.rho, order=plate.order, creases=plate.creases, rho_node=plate.rho_node,
                  kernel=plate.kernel, precision=shape_precision)
        self.faces = shape_functions(self.ctx, plate.faces.xy, **kw)
        self.fold_sets = []
        folds = []
        for f in plate.folds:
            L_ = shape_functions(self.ctx, f.left.xy, **kw)
            R_ = shape_functions(self.ctx, f.right.xy, **kw)
            self.fold_sets.append((L_, R_))
            folds.append({"left": L_, "right": R_, "weight": f.left.weight, "tangent": f.left.tangent,
                          "Kt": f.Kt, "theta0": f.theta0})
        self.fold_specs = folds
        # Point domains (GmshReader point elements), entity tag -> shape set, for
        # point supports and loads.
        self.point_sets = {tag: shape_functions(self.ctx, ps.xy, **kw) for tag, ps in plate.points.items()}
        self.asm = NonLinearAssembler(self.ctx, self.faces, plate.faces.weight, folds)
        A, B, D = abd_isotropic(plate.E, plate.nu, plate.thickness)
        self.asm.set_material(A, B, D)

    def shape_sets(self):
        """Every shape set of the model: faces, each fold's left and right, each point domain."""
        out = [self.faces]
        for L_, R_ in self.fold_sets:
            out += [L_, R_]
        return out + list(self.point_sets.values())

    def rebuild(self, creases):
        """SetupHelper::recomputeShapeFunctions (plate/SetupHelper.h:112-138) on the GPU:
        every shape set of the model recomputed in place for the cuts `creases`, the
        neighbour lists and the K pattern kept (they depend on the support radius only)."""
        for sh in self.shape_sets():
            sh.rebuild(creases)

    def assemble_system(self, x, flags=L.TANGENT | L.HINGE):
        return self.asm.assemble(x, flags)

    def assemble_internal_only(self, x, flags=L.HINGE):
        return self.asm.assemble(x, flags & ~L.TANGENT)[1]


class PlateBatch:
    """Independent plates of uneven size assembled as one problem: each plate's shape
    functions are built over its own nodes and creases, then stacked (concat_shapes) over
    the union of all nodes, so one assembler — one set of launches, or one graph launch —
    covers every plate's Gauss points. The union K is block diagonal: plate k owns dofs
    [3 o_k, 3 o_{k+1}) and the K values [outer[3 o_k], outer[3 o_{k+1}])."""

    def __init__(self, plates, ctx: Context | None = None):
        self.plates = list(plates)
        self.ctx = ctx or Context(0)
        p0 = self.plates[0]
        for p in self.plates:
            if (p.E, p.nu, p.thickness) != (p0.E, p0.nu, p0.thickness):
                raise ValueError("PlateBatch: every plate needs the same laminate (one material per assembler)")
        sizes = [len(p.node_xy) for p in self.plates]
        self.node_offset = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        faces, weights, folds, self._keep = [], [], [], []
        for k, p in enumerate(self.plates):
            self.ctx.set_nodes(p.node_xy)
            kw = dict(rho=p.rho, order=p.order, creases=p.creases, rho_node=p.rho_node, kernel=p.kernel)
            faces.append(shape_functions(self.ctx, p.faces.xy, **kw))
            weights.append(p.faces.weight)
            for f in p.folds:
                folds.append((k, f, shape_functions(self.ctx, f.left.xy, **kw),
                              shape_functions(self.ctx, f.right.xy, **kw)))
        self.node_xy = np.concatenate([p.node_xy for p in self.plates])
        self.ctx.set_nodes(self.node_xy)
        off = self.node_offset[:-1]
        self.faces = concat_shapes(self.ctx, faces, off)
        specs = []
        for k, f, Ls, Rs in folds:
            L_ = concat_shapes(self.ctx, [Ls], [off[k]])
            R_ = concat_shapes(self.ctx, [Rs], [off[k]])
            self._keep += [L_, R_]
            specs.append({"left": L_, "right": R_, "weight": f.left.weight, "tangent": f.left.tangent,
                          "Kt": f.Kt, "theta0": f.theta0})
        self.fold_specs = specs
        self.weight = np.concatenate(weights)
        self.asm = NonLinearAssembler(self.ctx, self.faces, self.weight, specs)
        self.asm.set_material(*abd_isotropic(p0.E, p0.nu, p0.thickness))
        outer, _ = self.asm.pattern()
        self.outer = outer
        self.n_gp = self.faces.n_gp

    def dofs(self, k):
        return slice(3 * int(self.node_offset[k]), 3 * int(self.node_offset[k + 1]))

    def k_values(self, k):
        return slice(int(self.outer[3 * self.node_offset[k]]), int(self.outer[3 * self.node_offset[k + 1]]))
