"""Adjoint of the plain FP64 step against central finite differences of the
same map (each step's iteration counts held at the recorded values), along
seeded random directions in the initial u, v, p and the lid profile.

The directions perturb the interior unknowns only: the wall-face velocities
are exactly 0, where the upwind selector of their momentum rows
(cj = 2 yeu u on a Cartesian grid) sits on its branch boundary, so a central
difference there straddles a kink of the map (and the boundary programs
overwrite those values anyway)."""
import dataclasses

import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver

pytestmark = pytest.mark.gpu

NORTH, VAR_U = 4, 1


def _setup(n, re, dt, mqiter, msorit, seed=11):
    case = deck.cavity(n, re, dt, solver="rb_sor")
    prm = dataclasses.replace(case.params, mqiter=mqiter, msorit=msorit)
    u, v, p = deck.perturbation_ic(case, seed)
    rng = np.random.default_rng(seed)
    p = p + 1e-3 * rng.normal(size=p.shape)
    p = np.asfortranarray(p)
    lid = np.ones(case.nx + 2) + 0.05 * np.sin(np.linspace(0, 3, case.nx + 2))
    return case, prm, (u, v, p), lid


def _interior(case):
    """Masks of the interior unknowns of u, v, p."""
    nx, ny = case.nx, case.ny
    mu = np.zeros((nx + 2, ny + 2), bool)
    mv = np.zeros_like(mu)
    mp = np.zeros_like(mu)
    mu[2:nx, 2:ny + 1] = True
    mv[2:nx + 1, 2:ny] = True
    mp[2:nx + 1, 2:ny + 1] = True
    return mu, mv, mp


def _objective(case, u, v, w):
    nx, ny = case.nx, case.ny
    return 0.5 * w * (np.sum(u[1:nx + 1, 2:ny + 1] ** 2) + np.sum(v[2:nx + 1, 1:ny + 1] ** 2))


def _forward(case, prm, fields, lid, counts, w):
    s = Solver.for_case(case, tuned=False)
    s.set_face_profile(1, 1, NORTH, VAR_U, lid)
    s.load_fields(*fields)
    s.step_counts(prm, counts)
    u, v, _ = s.store_fields()
    s.close()
    return _objective(case, u, v, w)


@pytest.mark.parametrize("nsteps,every,mqiter,msorit", [(1, 1, 1, 2), (1, 1, 3, 30), (3, 2, 4, 40), (5, 2, 20, 60)])
def test_adjoint_matches_finite_differences(nsteps, every, mqiter, msorit):
    """Along random interior directions (u0, v0, p0 and the lid profile
    together), the adjoint's directional derivative equals the central
    difference of the frozen-count map."""
    case, prm, fields, lid = _setup(32, 200.0, 0.004, mqiter, msorit)
    w = (1.0 / 32) ** 2
    s = Solver.for_case(case, tuned=False)
    s.set_face_profile(1, 1, NORTH, VAR_U, lid)
    s.load_fields(*fields)
    J, gu, gv, gp, gl, counts = s.adjoint(prm, nsteps, every, w, profile=(1, 1, NORTH, VAR_U),
                                          nprof=case.nx + 2)
    s.close()
    assert J == pytest.approx(_forward(case, prm, fields, lid, counts, w), rel=1e-14)
    rng = np.random.default_rng(7)
    eps = 1e-6
    masks = _interior(case)
    for _ in range(3):
        du, dv, dp = (np.asfortranarray(np.where(m, rng.normal(size=f.shape), 0.0)) for f, m in zip(fields, masks))
        dl = rng.normal(size=lid.shape)
        plus = [np.asfortranarray(f + eps * d) for f, d in zip(fields, (du, dv, dp))]
        minus = [np.asfortranarray(f - eps * d) for f, d in zip(fields, (du, dv, dp))]
        fd = (_forward(case, prm, plus, lid + eps * dl, counts, w) -
              _forward(case, prm, minus, lid - eps * dl, counts, w)) / (2 * eps)
        ad = np.sum(gu * du) + np.sum(gv * dv) + np.sum(gp * dp) + np.sum(gl * dl)
        assert ad == pytest.approx(fd, rel=1e-5, abs=100 * np.finfo(float).eps * abs(J) / eps), (ad, fd)


def test_lid_gradient_reaches_interior_after_two_steps():
    """The lid's ghost row enters the flow through the next step's momentum
    rows: one step leaves J independent of it, two do not; the adjoint's lid
    gradient equals finite differences per lid position."""
    case, prm, fields, lid = _setup(16, 100.0, 0.004, 6, 20)
    w = (1.0 / 16) ** 2
    res = {}
    for nsteps in (1, 2):
        s = Solver.for_case(case, tuned=False)
        s.set_face_profile(1, 1, NORTH, VAR_U, lid)
        s.load_fields(*fields)
        res[nsteps] = s.adjoint(prm, nsteps, 1, w, profile=(1, 1, NORTH, VAR_U), nprof=case.nx + 2)
        s.close()
    assert not np.any(res[1][4])
    J, gu, gv, gp, gl, counts = res[2]
    assert np.any(gl)
    eps = 1e-6
    for i in (2, case.nx // 2, case.nx):
        dl = np.zeros_like(lid)
        dl[i] = 1.0
        fd = (_forward(case, prm, fields, lid + eps * dl, counts, w) -
              _forward(case, prm, fields, lid - eps * dl, counts, w)) / (2 * eps)
        # a central difference resolves J only to about its rounding over 2 eps
        assert gl[i] == pytest.approx(fd, rel=1e-5, abs=100 * np.finfo(float).eps * abs(J) / eps), (i, gl[i], fd)


@pytest.mark.parametrize("n,re,dt,mqiter,msorit,nsteps,every", [(16, 100.0, 0.004, 6, 20, 3, 2),
                                                                  (64, 400.0, 0.002, 8, 60, 20, 5)])
def test_adjoint_matches_reference_finite_differences(n, re, dt, mqiter, msorit, nsteps, every):
    """The GPU adjoint against central differences of the CPU reference
    restatement (the oracle, bit-identical to the GPU forward), run step by
    step with the same frozen counts: a 16x16 cavity over 3 steps and a
    64x64 cavity over 20 steps with checkpoints every 5."""
    import oracle as O
    case, prm, fields, lid = _setup(n, re, dt, mqiter, msorit)
    case.regions.profiles[(1, 1, NORTH, VAR_U)] = lid
    w = (1.0 / n) ** 2
    s = Solver.for_case(case, tuned=False)
    s.load_fields(*fields)
    J, gu, gv, gp, gl, counts = s.adjoint(prm, nsteps, every, w, profile=(1, 1, NORTH, VAR_U),
                                          nprof=case.nx + 2)
    s.close()

    def ref_J(flds, lidv):
        case.regions.profiles[(1, 1, NORTH, VAR_U)] = lidv
        r = O.OracleRun(case, fields={"u": flds[0], "v": flds[1], "p": flds[2]}, cold_start=False)
        for m, ns in counts:
            r._ps = O.Oracle.params_struct(dataclasses.replace(prm, mqiter=int(m), qtol=-1.0,
                                                               msorit=int(ns), sortol=-1.0))
            r.step(1)
        return _objective(case, r.f["u"], r.f["v"], w)

    assert ref_J(fields, lid) == pytest.approx(J, rel=1e-13)
    rng = np.random.default_rng(5)
    eps = 1e-6
    masks = _interior(case)
    du, dv, dp = (np.where(m, rng.normal(size=f.shape), 0.0) for f, m in zip(fields, masks))
    dl = rng.normal(size=lid.shape)
    fd = (ref_J([f + eps * d for f, d in zip(fields, (du, dv, dp))], lid + eps * dl) -
          ref_J([f - eps * d for f, d in zip(fields, (du, dv, dp))], lid - eps * dl)) / (2 * eps)
    ad = np.sum(gu * du) + np.sum(gv * dv) + np.sum(gp * dp) + np.sum(gl * dl)
    assert ad == pytest.approx(fd, rel=1e-5, abs=100 * np.finfo(float).eps * abs(J) / eps)


def test_autograd_wrapper():
    import torch
    from wolfd2_gb300.autograd import KineticEnergy
    case, prm, fields, lid = _setup(16, 100.0, 0.004, 6, 20)
    w = (1.0 / 16) ** 2
    s = Solver.for_case(case, tuned=False)
    u0 = torch.tensor(np.ascontiguousarray(fields[0].T)).T.requires_grad_()
    v0 = torch.tensor(np.ascontiguousarray(fields[1].T)).T.requires_grad_()
    lt = torch.tensor(lid, requires_grad=True)
    p0 = torch.tensor(np.ascontiguousarray(fields[2].T)).T
    J = KineticEnergy.apply(u0, v0, lt, s, prm, 2, 1, w, p0)
    J.backward()
    s.load_fields(*fields)
    s.set_face_profile(1, 1, NORTH, VAR_U, lid)
    J2, gu, gv, _, gl, _ = s.adjoint(prm, 2, 1, w, profile=(1, 1, NORTH, VAR_U), nprof=case.nx + 2)
    s.close()
    # J and the gradients are sums of FP64 atomics: equal up to their order
    assert float(J) == pytest.approx(J2, rel=1e-13)
    for g, ref in ((u0.grad, gu), (v0.grad, gv), (lt.grad, gl)):
        assert np.allclose(g.numpy(), ref, rtol=1e-11, atol=1e-12 * np.max(np.abs(ref)))


@pytest.mark.parametrize("outlet", ["mc", "fd"])
def test_channel_adjoint_inflow_profile(outlet):
    """Channel with a per-row inflow profile and an outlet (VelOutflowBCs
    inside every Q-L iteration): gradient with respect to the initial fields
    and the inflow profile against central differences.  The start is the
    flow after two steps: the initial field has v = 0 everywhere, where every
    v-driven upwind selector sits on its branch point."""
    WEST = 1
    case = deck.channel_inflow(48, 16, 500.0, 0.004, seed=3, length=3.0, outlet=outlet)
    prm = dataclasses.replace(case.params, mqiter=8, msorit=40)
    s = Solver.for_case(case, tuned=False)
    s.load_fields(*deck.channel_ic(case))
    s.step(prm, 2)
    fields = s.store_fields()
    s.close()
    prof = case.regions.profiles[(1, 1, WEST, VAR_U)].copy()
    w = (1.0 / 16) ** 2
    s = Solver.for_case(case, tuned=False)
    s.load_fields(*fields)
    J, gu, gv, gp, gl, counts = s.adjoint(prm, 3, 2, w, profile=(1, 1, WEST, VAR_U), nprof=case.ny + 2)
    s.close()
    assert np.any(gl)

    def J_at(flds, pr):
        s = Solver.for_case(case, tuned=False)
        s.set_face_profile(1, 1, WEST, VAR_U, pr)
        s.load_fields(*[np.asfortranarray(f) for f in flds])
        s.step_counts(prm, counts)
        u, v, _ = s.store_fields()
        s.close()
        return _objective(case, u, v, w)

    assert J_at(fields, prof) == pytest.approx(J, rel=1e-13)
    rng = np.random.default_rng(9)
    eps = 1e-6
    masks = _interior(case)
    for _ in range(2):
        du, dv, dp = (np.where(m, rng.normal(size=f.shape), 0.0) for f, m in zip(fields, masks))
        dl = np.zeros_like(prof)
        dl[2:case.ny + 1] = rng.normal(size=case.ny - 1)
        fd = (J_at([f + eps * d for f, d in zip(fields, (du, dv, dp))], prof + eps * dl) -
              J_at([f - eps * d for f, d in zip(fields, (du, dv, dp))], prof - eps * dl)) / (2 * eps)
        ad = np.sum(gu * du) + np.sum(gv * dv) + np.sum(gp * dp) + np.sum(gl * dl)
        assert ad == pytest.approx(fd, rel=1e-5, abs=100 * np.finfo(float).eps * abs(J) / eps), (ad, fd)
