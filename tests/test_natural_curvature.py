"""Natural curvature (Kinematics::NaturalCurvature, plate/Kinematics.h:21-45; set from the
config's "natural_curvature" band, main.cpp:83-95): the elastic bending strain
E1_el = E1 + kappa_bar(X) replaces E1 in the constitutive law, so it changes N, M, the
residual, the tangent's resultants and the bending energy, not the strain operators.

CPU (oracle): the restated field's formula, the reference's TangentCheck (K v against
central differences of F, < 1e-6) and F = dE/dx with the field active, and a flat plate
that the band alone loads (mountain and valley opposite). GPU (through the C ABI): the
FP64 and mixed assembly, the energies and the point state against the oracle on the same
shape functions (FP64 1e-13, mixed residual 1e-12 and tangent 1e-5), the refusals, and
that switching it off restores the plain results.
"""
import math

import numpy as np
import pytest

from curvami_gb300 import synth
from oracle import Oracle

BAND = {"x0": 3.0, "width": 1.0, "angle_deg": 30.0, "sense": "mountain"}


@pytest.fixture(scope="module")
def o():
    return Oracle()


def kappa_ref(X, nc):
    """Kinematics.h:25-34: sign * theta0 * exp(-((X - x0) / w)^2) / (sqrt(pi) w)."""
    sign = -1.0 if nc["sense"] == "mountain" else 1.0
    t = (np.asarray(X) - nc["x0"]) / nc["width"]
    return sign * math.radians(nc["angle_deg"]) * np.exp(-t * t) / (math.sqrt(math.pi) * nc["width"])


class Plate:
    """A 13 x 13 plate (h = 0.5) with a straight crease and the oracle's shape functions."""

    def __init__(self, o):
        self.o = o
        self.p = p = synth.square_plate(13, 0.5, 3, jitter=0.05, seed=71, crease="row", Kt=1e-3)
        ptr, idx, s = o.frnn(p.node_xy, p.faces.xy, p.rho)
        psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, p.faces.xy, ptr, idx, s, p.rho, p.order, p.creases)
        assert rc == 0
        self.sh = dict(ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi)
        outer, inner, col_ptr, col_nodes, mp = o.pattern(p.n_nodes, ptr, idx, [])
        self.outer, self.inner, self.mp = outer, inner, mp
        self.A, self.B, self.D = o.abd(p.E, p.nu, p.thickness)

    def assemble(self, x, want_K=True):
        s = self.sh
        return self.o.update_stiffness(self.p.n_nodes, self.p.faces.weight, s["ptr"], s["idx"], s["dpsi"],
                                       s["ddpsi"], self.outer, self.mp, x, self.A, self.B, self.D, want_K=want_K,
                                       gp_xy=self.p.faces.xy)

    def energy(self, x):
        s = self.sh
        em, eb = self.o.strain_energies(self.p.faces.weight, s["ptr"], s["idx"], s["dpsi"], s["ddpsi"], x,
                                        self.A, self.B, self.D, gp_xy=self.p.faces.xy)
        return em + eb


def sym_apply(K_vals, outer, inner, v):
    """selfadjointView<Upper> * v for the block-upper CSC K: only the scalar upper triangle is
    read (the diagonal blocks are stored whole)."""
    import scipy.sparse as sp

    n = len(outer) - 1
    U = sp.triu(sp.csc_matrix((K_vals, inner, outer), shape=(n, n)))
    return U @ v + sp.triu(U, k=1).T @ v


def test_field_formula_and_kinematics(o):
    pl = Plate(o)
    o.set_natural_curvature(BAND)
    try:
        x = 0.05 * synth.fourier_field(pl.p.node_xy, np.random.default_rng(5), lam=(2.0, 6.0))
        s = pl.sh
        for g in (0, 100, 400):
            k = o.kinematics(g, s["ptr"], s["idx"], s["dpsi"], s["ddpsi"], x, X=pl.p.faces.xy[g])
            kb = kappa_ref(pl.p.faces.xy[g, 0], BAND)
            assert abs(k[28] - (k[25] + kb)) <= 1e-15 * max(1.0, abs(kb))
            assert k[29] == k[26] and k[30] == k[27]
    finally:
        o.set_natural_curvature(None)


def test_tangent_and_energy_consistency(o):
    pl = Plate(o)
    rng = np.random.default_rng(6)
    x = 0.05 * synth.fourier_field(pl.p.node_xy, rng, lam=(2.0, 6.0))
    o.set_natural_curvature(BAND)
    try:
        K, F = pl.assemble(x)
        for _ in range(3):                       # TangentCheck (main.cpp:651-710)
            v = rng.uniform(-1.0, 1.0, len(x)) * 0.05 * np.abs(x).max()
            h = 1e-6
            Fp = pl.assemble(x + h * v, want_K=False)[1]
            Fm = pl.assemble(x - h * v, want_K=False)[1]
            fd = (Fp - Fm) / (2 * h)
            Kv = sym_apply(K, pl.outer, pl.inner, v)
            assert np.abs(fd - Kv).max() / np.abs(Kv).max() < 1e-6
        v = rng.standard_normal(len(x))            # F = dE/dx
        h = 1e-6 * np.abs(x).max() / np.abs(v).max()
        dE = (pl.energy(x + h * v) - pl.energy(x - h * v)) / (2 * h)
        assert abs(dE - F @ v) <= 1e-6 * abs(F @ v)
    finally:
        o.set_natural_curvature(None)


def test_band_loads_the_flat_plate(o):
    pl = Plate(o)
    x = np.zeros(3 * pl.p.n_nodes)
    F0 = pl.assemble(x, want_K=False)[1]
    assert np.abs(F0).max() == 0.0
    out = {}
    for sense in ("mountain", "valley"):
        o.set_natural_curvature(dict(BAND, sense=sense))
        out[sense] = pl.assemble(x, want_K=False)[1]
    o.set_natural_curvature(None)
    assert np.abs(out["mountain"]).max() > 0.0
    assert np.allclose(out["mountain"], -out["valley"], rtol=0, atol=1e-15 * np.abs(out["mountain"]).max())
    # flat: E1 = 0, so M = D kappa_bar and only bending terms act (no in-plane force)
    assert np.abs(out["mountain"].reshape(-1, 3)[:, :2]).max() <= 1e-14 * np.abs(out["mountain"]).max()


# ---- GPU ---------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def gpu():
    import __graft_entry__ as ge

    ge.build()
    import curvami_gb300 as cg

    ctx = cg.Context(0)
    p = synth.square_plate(21, 0.5, 4, jitter=0.1, seed=72, crease="arc", Kt=1e-3)
    ctx.set_nodes(p.node_xy)
    model = cg.PlateModel(p, ctx)
    return cg, ctx, p, model


@pytest.mark.gpu
def test_gpu_assembly_energies_and_state_against_oracle(o, gpu):
    cg, ctx, p, model = gpu
    from curvami_gb300 import export

    x = 0.1 * synth.fourier_field(p.node_xy, np.random.default_rng(73), lam=(3.0, 12.0))
    sh = model.faces.download()
    outer, inner, col_ptr, col_nodes, mp = o.pattern(p.n_nodes, sh["ptr"], sh["idx"], [])
    A, B, D = o.abd(p.E, p.nu, p.thickness)
    asm = cg.NonLinearAssembler(ctx, model.faces, p.faces.weight)
    asm.set_material(*cg.abd_isotropic(p.E, p.nu, p.thickness))
    K_plain, F_plain = asm.assemble(x, cg.TANGENT)
    ctx.set_natural_curvature(BAND)
    o.set_natural_curvature(BAND)
    rel = lambda a, b: float(np.abs(a - b).max() / np.abs(b).max())  # noqa: E731
    try:
        Ko, Fo = o.update_stiffness(p.n_nodes, p.faces.weight, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"],
                                    outer, mp, x, A, B, D, gp_xy=p.faces.xy)
        K, F = asm.assemble(x, cg.TANGENT)
        assert rel(K, Ko) < 1e-13 and rel(F, Fo) < 1e-13
        assert rel(F, F_plain) > 1e-6          # the band changes the residual
        Km, Fm = asm.assemble(x, cg.TANGENT | cg.MIXED)
        assert rel(Fm, Fo) < 1e-12 and rel(Km, Ko) < 1e-5
        em, eb, _ = asm.energies(x)
        emo, ebo = o.strain_energies(p.faces.weight, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"], x, A, B, D,
                                     gp_xy=p.faces.xy)
        assert abs(em - emo) <= 1e-12 * abs(emo) and abs(eb - ebo) <= 1e-12 * abs(ebo)
        st = export.point_state(ctx, model.faces, x, A, B, D)
        for g in (0, 333, 1000):
            k = o.kinematics(g, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"], x, X=p.faces.xy[g])
            assert np.allclose(st[g, 24:27], k[25:28], rtol=0, atol=1e-12 * max(1.0, np.abs(k[25:28]).max()))
            e0 = np.array([k[22], k[23], 2 * k[24]])
            e1 = np.array([k[28], k[29], 2 * k[30]])
            M = np.asarray(B).reshape(3, 3).T @ e0 + np.asarray(D).reshape(3, 3) @ e1
            assert np.allclose(st[g, 30:33], M, rtol=0, atol=1e-12 * np.abs(M).max())
    finally:
        ctx.set_natural_curvature(None)
        o.set_natural_curvature(None)
    K2, F2 = asm.assemble(x, cg.TANGENT | cg.DETERMINISTIC)
    K3, F3 = asm.assemble(x, cg.TANGENT | cg.DETERMINISTIC)
    assert np.array_equal(F2, F3)
    assert np.abs(F2 - F_plain).max() <= 1e-13 * np.abs(F_plain).max()


@pytest.mark.gpu
def test_gpu_refusals(gpu):
    cg, ctx, p, model = gpu
    sh = model.faces.download()
    faces_h = cg.shape_from_host(ctx, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"], sh["psi"])
    asm = cg.NonLinearAssembler(ctx, faces_h, p.faces.weight)
    asm.set_material(*cg.abd_isotropic(p.E, p.nu, p.thickness))
    x = np.zeros(3 * p.n_nodes)
    ctx.set_natural_curvature(BAND)
    try:
        with pytest.raises(cg.CGBError) as e:
            asm.assemble(x, cg.TANGENT)
        assert e.value.code == 1 and "reference coordinates" in str(e.value)
        with pytest.raises(cg.CGBError):
            ctx.set_natural_curvature(dict(BAND, width=0.0))
    finally:
        ctx.set_natural_curvature(None)
    asm.assemble(x, cg.TANGENT)   # fine again once it is off
