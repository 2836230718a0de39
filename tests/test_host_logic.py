"""Host-side logic that needs no GPU: the ensemble packing
(gb300dem.ensemble.pack) and the elastoplastic bond-table mapping
(gb300dem.workloads.elastoplastic_bond_params).

pack() must keep every system's atoms and coordinates unchanged, give system
k the atom type k+1 and its own material on the table diagonal, offset the
tags so that they stay unique, and turn each system's floor into a per-type
plane at its own height; it must refuse systems the ensemble cannot hold.

The bond mapping must give the reference's bond/nonlinear tables
(src/cohesion_model_bond_nonlinear.h:582-615, :666-872) the properties its
docstring states for a bilinear material: elastic unloading (Ku = Kc = E/L0,
G/L0 for shear and twist), the secant at the reference strain as the loading
stiffness, the bilinear material's permanent set after unloading from that
strain, and the same for the compression law's sqrt form.
"""
import math

import numpy as np
import pytest

from gb300dem import ensemble, workloads


def _systems(nsys=3):
    out = []
    for k in range(nsys):
        c = workloads.lattice_case(seed=10 + k, nx=4, ny=4, nz=2 + k, spacing=2.2e-3, radius=(0.9e-3, 1.1e-3),
                                   E=(1e6 * (k + 1),), rest=((0.5 + 0.1 * k,),), frict=((0.2 + 0.1 * k,),),
                                   plane_z=0.001 * k, jitter=1e-5, zhi=0.05)
        out.append(c)
    return out


def test_pack_keeps_each_system_and_separates_them():
    systems = _systems()
    case, layout = ensemble.pack(systems)
    assert case["ntypes"] == len(systems) == layout["nsys"] == case["ensemble"]
    a = case["atoms"]
    assert layout["counts"] == [len(s["atoms"]["tag"]) for s in systems]
    assert len(a["tag"]) == sum(layout["counts"])
    assert len(np.unique(a["tag"])) == len(a["tag"])  # tags unique across systems
    start = 0
    for k, s in enumerate(systems):
        n = layout["counts"][k]
        sl = slice(start, start + n)
        assert np.all(a["type"][sl] == k + 1)
        for name in ("x", "v", "omega", "radius", "rmass"):
            assert np.array_equal(a[name][sl], s["atoms"][name]), (k, name)
        assert np.array_equal(a["tag"][sl], s["atoms"]["tag"] + layout["offsets"][k])
        for tab in ("Yeff", "Geff", "betaeff", "coeffFrict", "coeffRestLog"):
            assert case[tab][k + 1, k + 1] == np.asarray(s[tab])[1, 1], (k, tab)
        start += n
    # the floors: one per-type plane list, each system's at its own height
    assert case["planes"] == []
    axis, heights, _ = case["planes_per_type"][0]
    assert axis == systems[0]["planes"][0][0]
    for k, s in enumerate(systems):
        assert heights[k + 1] == pytest.approx(float(s["planes"][0][1]))


def test_pack_refuses_what_an_ensemble_cannot_hold():
    with pytest.raises(ValueError):
        ensemble.pack([])
    a, b = _systems(2)
    b = dict(b, dt=2 * b["dt"])
    with pytest.raises(ValueError):
        ensemble.pack([a, b])
    a, b = _systems(2)
    b = dict(b, planes=[])
    with pytest.raises(ValueError):
        ensemble.pack([a, b])
    a, b = _systems(2)
    b = dict(b, meshes=[dict(nodes=np.zeros((1, 3, 3)), wall_type=1, rolling=0)])
    with pytest.raises(ValueError):
        ensemble.pack([a, b])


def _table(params, name):
    k = workloads.BOND_TABLES.index(name)
    t = params["tables"][k]
    return float(t[1, 1])


@pytest.mark.parametrize("E,eps_y,h", [(1e9, 0.01, 0.1), (5e8, 0.02, 0.3), (2e9, 0.005, 0.0)])
def test_elastoplastic_bond_tables(E, eps_y, h):
    r, lam, nu, f = 0.5e-3, 0.5, 0.3, 2.0
    p = workloads.elastoplastic_bond_params(2, [1], E=E, yield_strain=eps_y, hardening=h, radius=r, lam=lam,
                                            nu=nu, ref_strain_factor=f)
    L0, A, G = 2 * r, math.pi * (lam * r) ** 2, E / (2 * (1 + nu))
    eps_r = f * eps_y
    sig = E * (eps_y + h * (eps_r - eps_y))  # the bilinear stress at the reference strain
    K, Ku, Kc = (_table(p, "stiffnessPerUnitArea" + n) for n in ("K_fn2", "Ku_fn2", "Kc_fn2"))
    # elastic unloading and reloading past the origin
    assert Ku == pytest.approx(E / L0) and Kc == pytest.approx(E / L0)
    # loading along the secant: the stress at eps_r is the bilinear one
    assert K * L0 * eps_r == pytest.approx(sig)
    # unloading from eps_r along Ku leaves the bilinear material's permanent set
    d_r = eps_r * L0
    d_set = d_r - K * d_r / Ku
    assert d_set / L0 == pytest.approx(eps_r - sig / E)
    # compression: K_fn1 sqrt(d) reaches A sigma at eps_r, and its unloading
    # along Ku_fn1 sqrt(.) leaves the same permanent set
    K1, Ku1, Kc1 = (_table(p, "stiffnessPerUnitArea" + n) for n in ("K_fn1", "Ku_fn1", "Kc_fn1"))
    assert K1 * math.sqrt(d_r) == pytest.approx(A * sig)
    assert (1 - K1 / Ku1) ** 2 == pytest.approx(1 - sig / (E * eps_r))
    assert Kc1 == Ku1
    # shear and twist take G, bend E; their loading stiffnesses the same secant
    assert _table(p, "stiffnessPerUnitAreaK_ft") == pytest.approx(G / L0)
    assert _table(p, "stiffnessPerUnitAreaKu_tn") == pytest.approx(G / L0)
    assert _table(p, "stiffnessPerUnitAreaK_tn") == pytest.approx(sig / (E * eps_r) * G / L0)
    assert _table(p, "stiffnessPerUnitAreaKu_tt") == pytest.approx(E / L0)
    assert _table(p, "stiffnessPerUnitAreaK_tt") == pytest.approx(K)
    # the bond radius multiplier only between the bonded types
    rm = p["tables"][workloads.BOND_TABLES.index("radiusMultiplierBondnonlinear")]
    assert rm[1, 1] == lam and rm[1, 2] == 0.0 and rm[2, 2] == 0.0
