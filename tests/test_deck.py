"""Host-side case setup: the boundary_conditions grammar, SetUpBCs passes,
restart records and deck writers."""
import os

import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.deck import BM_INLET, BM_INTERN, BM_OUTLT1, BM_OUTLT2, BM_WALL1, BM_WALL2


def test_cavity_tables():
    c = deck.cavity(64, 100.0, 0.005)
    r = c.regions
    assert (r.n_i, r.n_j) == (1, 1)
    assert [r.border(1, 1, f) for f in (1, 2, 3, 4)] == [1, 65, 1, 65]
    assert [r.btype(1, 1, f) for f in (1, 2, 3, 4)] == [BM_WALL1] * 4
    assert r.dBCVal[0, 0, deck.NORTH - 1, deck.VAR_U - 1] == 1.0
    assert c.params.re == 100.0 and c.params.npsolver == 1 and c.params.lcartes == 1


def test_region_borders_and_consistency():
    text = """number_of_regions 3 2
i_borders 10 20
j_borders 8
wall 1 1 east no_stress     # internal wall between (1,1) and (2,1)
inlet 2 2 south nv 0.5
inlet 1 2 south nv 0.25
outlet 3 1 east fd p 2.0
outlet 3 2 east
blockage 2 1"""
    r = deck.parse_bc_section(text, 33, 17)
    assert [r.border(2, 2, f) for f in (1, 2, 3, 4)] == [10, 20, 8, 17]
    assert r.btype(3, 1, deck.EAST) == BM_OUTLT1 and r.btype(3, 2, deck.EAST) == BM_OUTLT2
    # blockage makes its faces and the neighbours' shared faces no-slip walls
    assert r.btype(1, 1, deck.EAST) == BM_WALL1 and r.btype(3, 1, deck.WEST) == BM_WALL1
    # a later blockage line overrides the earlier inlet on its shared face
    assert r.btype(2, 2, deck.SOUTH) == BM_WALL1 and r.btype(2, 1, deck.NORTH) == BM_WALL1
    # an inlet propagates to the neighbour's shared face (bound_cond.f:210-223)
    assert r.btype(1, 1, deck.NORTH) == BM_INLET
    assert r.dBCVal[0, 1, deck.SOUTH - 1, deck.VAR_V - 1] == 0.25
    assert r.dBCVal[2, 0, deck.EAST - 1, deck.VAR_P - 1] == 2.0
    assert r.btype(2, 2, deck.WEST) == BM_INTERN


@pytest.mark.parametrize("bad", [
    "number_of_regions 2 1\ni_borders 1\nj_borders\n",          # border < 2
    "number_of_regions 1 1\ni_borders\nj_borders\nwall 1 1 up\n",
    "number_of_regions 1 1\ni_borders\nj_borders\nwhatever 1 1\n",
    "i_borders 3\n",
])
def test_rejected_decks(bad):
    with pytest.raises(deck.DeckError):
        deck.parse_bc_section(bad, 17, 17)


def test_restart_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    flds = [np.asfortranarray(rng.normal(size=(10, 8))) for _ in range(8)]
    path = str(tmp_path / "r.rst")
    deck.write_restart(path, 7, 0.35, 8, 6, flds)
    k, t, nx, ny, back = deck.read_restart(path)
    assert (k, t, nx, ny) == (7, 0.35, 8, 6)
    for a, b in zip(flds, back):
        assert np.array_equal(a, b)


def test_deck_files(tmp_path):
    c = deck.channel(16, 8, 500.0, 1e-3)
    deck.write_deck(str(tmp_path / "input.dat"), c, nts=3)
    deck.write_grid_plot3d(str(tmp_path / "grid.xyz"), c.x, c.y)
    deck.write_fluid_table(str(tmp_path / "fluidprop.dat"), 1.0, 0.002)
    txt = open(tmp_path / "input.dat").read()
    assert "ppe_solver rb_sor" in txt and "outlet 1 1 east fd" in txt
    first = open(tmp_path / "grid.xyz").readline().split()
    assert first == ["17", "9"]
    sec = txt.split("section boundary_conditions")[1].split("end section")[0]
    r = deck.parse_bc_section(sec, c.nx, c.ny)
    assert np.array_equal(r.nMomBdTp, c.regions.nMomBdTp)


def test_thermal_keywords():
    """parse.f's thermal keywords: defaults (adiabatic outer walls,
    interfaces inside), temperatures on walls scaled to (T - tref)/(tmax -
    tref), fixed-temperature blocks with their neighbours' faces, heat
    generation regions and the coinciding-face pairing of SetUpBCs."""
    from wolfd2_gb300.deck import (BT_HTFLUX, BT_INTERN, BT_TEMPER, RT_HEATGN, RT_TEMPER, VAR_T,
                                   heat_sources, parse_bc_section)
    text = ("number_of_regions 3 2\n i_borders 10 20\n j_borders 8\n"
            "wall 1 1 west t 350\n blockage 2 1 temper 320\n"
            "heat_generation_region 3 2 5.0\n fixed_temperature_wall 1 2 north 330\n"
            "heat_flux_wall 3 1 east\n")
    r = parse_bc_section(text, 31, 17, tref=300.0, tmax=400.0)
    th = r.thermal
    assert th.nTemBdTp[0, 0, deck.WEST - 1] == BT_TEMPER
    assert r.dBCVal[0, 0, deck.WEST - 1, VAR_T - 1] == (350.0 - 300.0) / 100.0
    assert th.nTRgType[1, 0] == RT_TEMPER and th.dTRgVal[1, 0] == 0.2
    assert (th.nTemBdTp[1, 0, :] == BT_TEMPER).all()
    # the block's neighbours see its temperature on their coinciding faces
    assert th.nTemBdTp[0, 0, deck.EAST - 1] == BT_TEMPER and th.nTemBdTp[2, 0, deck.WEST - 1] == BT_TEMPER
    assert th.nTemBdTp[1, 1, deck.SOUTH - 1] == BT_TEMPER
    assert r.dBCVal[1, 1, deck.SOUTH - 1, VAR_T - 1] == 0.2
    assert th.nTRgType[2, 1] == RT_HEATGN and th.dTRgVal[2, 1] == 5.0
    assert th.nTemBdTp[0, 1, deck.NORTH - 1] == BT_TEMPER
    assert th.nTemBdTp[2, 0, deck.EAST - 1] == BT_HTFLUX
    # interfaces stay interfaces, outer walls default to adiabatic
    assert th.nTemBdTp[0, 1, deck.EAST - 1] == BT_INTERN
    assert th.nTemBdTp[2, 1, deck.NORTH - 1] == BT_HTFLUX
    heat_sources(r, 1.0, 300.0, 400.0, 2.0, 10.0)
    assert th.dHGSTval[2, 1] == 5.0 / (10.0 * 2.0 * 100.0)


def test_plot3d_solution_layout(tmp_path):
    """SaveStdVarsP3D's unformatted solution file: (nx, ny, nVars), then
    p, u, v, w = 0 (and t) over i = 1..nx, j = 1..ny, i fastest."""
    import numpy as np
    nx, ny = 7, 5
    rng = np.random.default_rng(0)
    u, v, p, t = (np.asfortranarray(rng.normal(size=(nx + 2, ny + 2))) for _ in range(4))
    pre = str(tmp_path / "snap")
    deck.write_plot3d_solution(pre, nx, ny, u, v, p, t)
    n1, n2, f = deck.read_plot3d_solution(pre + ".qqq")
    assert (n1, n2, f.shape[2]) == (nx, ny, 5)
    for l, a in enumerate((p, u, v, np.zeros_like(p), t)):
        assert np.array_equal(f[:, :, l], a[1:nx + 1, 1:ny + 1])
    raw = open(pre + ".qqq", "rb").read()
    assert np.frombuffer(raw[:4], "<i4")[0] == 12 and len(raw) == 4 + 12 + 4 + 4 + nx * ny * 5 * 8 + 4
    assert open(pre + ".nam").read().splitlines()[-1] == " Complete Temperature"


def test_read_deck_round_trip(tmp_path):
    """A deck written by write_deck (with its grid and fluid files) reads back
    into the same case: ReadParam's scaling gives the same dk and Re, the grid
    and the region tables are the same."""
    c = deck.channel(16, 8, 500.0, 1e-3, solver="par_rb_sor")
    deck.write_deck(str(tmp_path / "input.dat"), c, nts=3)
    deck.write_grid_plot3d(str(tmp_path / "grid.xyz"), c.x, c.y)
    deck.write_fluid_table(str(tmp_path / "fluidprop.dat"), 1.0, 1.0 / c.params.re)
    r = deck.read_deck(str(tmp_path / "input.dat"))
    assert (r.nx, r.ny) == (c.nx, c.ny)
    assert np.array_equal(r.x, c.x) and np.array_equal(r.y, c.y)
    for k in ("dk", "npsolver", "msorit", "sortol", "sorrel", "mqiter", "qtol", "lcartes"):
        assert getattr(r.params, k) == getattr(c.params, k), k
    assert r.params.re == pytest.approx(c.params.re, rel=1e-15)
    assert r.params.nts == 3
    for k in ("nRegBrd", "nRegType", "nMomBdTp", "dBCVal"):
        assert np.array_equal(getattr(r.regions, k), getattr(c.regions, k)), k
    assert r.thermal is None


def test_read_deck_thermal_and_fluid_interpolation(tmp_path):
    """thermal_energy / buoyancy decks: Pe = Re Pr and Fr from the reference
    quantities, the fluid row interpolated at ref_temperature, temperatures
    scaled to (T - tref)/(tmax - tref), heat sources scaled."""
    (tmp_path / "grid.xyz").write_text("")
    c = deck.cavity(8, 100.0, 0.01)
    deck.write_grid_plot3d(str(tmp_path / "grid.xyz"), c.x, c.y)
    (tmp_path / "fluid.dat").write_text(
        "# two fluids\nfluid water\n250 2.0 4.0 0.02 0.6 7.0\n350 2.0 4.0 0.02 0.6 7.0\nend\n"
        "fluid air01 gasconstant 287.0\n280 1.2 1000 0.010 0.025 0.70\n320 1.0 1000 0.012 0.027 0.72\nend\n")
    (tmp_path / "input.dat").write_text(
        "section input_parameters\n grid_file grid.xyz cartesian_grid\n thermal_energy\n buoyancy\n"
        " time_step_size 0.02\n ref_length 2.0\n ref_velocity 0.5\n ref_temperature 300\n"
        " max_ref_temperature 400\n fluid_prop_file fluid.dat\n max_me_iter 3\n me_tolerance 1d-6\n"
        " filter_t 8.0\n ppe_solver rb_sor\nend section\n\n"
        "section boundary_conditions\n number_of_regions 1 1\n i_borders\n j_borders\n"
        " wall 1 1 west t 350\n heat_generation_region 1 1 5.0\nend section\n")
    r = deck.read_deck(str(tmp_path / "input.dat"))
    rho, mu, k, pr = 1.1, 0.011, 0.026, 0.71      # the rows at 300 K
    assert r.params.dk == pytest.approx(0.02 * 0.5 / 2.0)
    assert r.params.re == pytest.approx(2.0 * 0.5 / (mu / rho), rel=1e-12)
    assert r.params.fr == pytest.approx(0.25 / (2.0 * 9.81))
    tp = r.tparams
    assert (tp.nthermen, tp.neqstate, tp.nmeiter, tp.nfiltt) == (1, 1, 3, 1)
    assert tp.dmeittol == 1e-6 and tp.fpt == 8.0 and tp.rconst == 287.0
    assert tp.pe == pytest.approx(r.params.re * pr, rel=1e-12)
    assert r.regions.dBCVal[0, 0, deck.WEST - 1, deck.VAR_T - 1] == pytest.approx(0.5)
    assert r.thermal.dHGSTval[0, 0] == pytest.approx(5.0 * 4.0 / (tp.pe * k * 100.0), rel=1e-12)
    assert r.x.max() == pytest.approx(c.x.max() / 2.0)


def test_read_deck_small_scale_keywords(tmp_path):
    """small_scale and the atd_* keywords (src/parse.f:342-344, 491-620)
    become the case's SmallScale parameters; unset ones keep parse.f's
    defaults, and the case carries thermal tables for the model."""
    c = deck.cavity(8, 100.0, 0.01)
    deck.write_grid_plot3d(str(tmp_path / "grid.xyz"), c.x, c.y)
    (tmp_path / "fluid.dat").write_text(
        "fluid air01 gasconstant 287.0\n280 1.2 1000 0.010 0.025 0.70\n320 1.0 1000 0.012 0.027 0.72\nend\n")
    (tmp_path / "input.dat").write_text(
        "section input_parameters\n grid_file grid.xyz cartesian_grid\n small_scale\n"
        " time_step_size 0.01\n ref_temperature 300\n fluid_prop_file fluid.dat\n"
        " atd_cu0 0.7\n atd_bnumcrit 12.5\n atd_rmapmax 0.9\n atd_ppe_solver rb_lsor\n"
        " atd_max_sor_iter 500\n atd_sor_tolerance 1d-9\n atd_filter_t 250\nend section\n\n"
        "section boundary_conditions\n number_of_regions 1 1\n i_borders\n j_borders\n"
        " wall 1 1 north tv 1.0\nend section\n")
    r = deck.read_deck(str(tmp_path / "input.dat"))
    a = r.atd
    assert (a.cu0, a.bnumc, a.rmax, a.msorit, a.sortol, a.fpt) == (0.7, 12.5, 0.9, 500, 1e-9, 250.0)
    assert a.npsolver == deck.PPE_SOLVERS["rb_lsor"]
    assert (a.tscoef, a.hscoef, a.temcoef, a.rlc, a.fpu, a.sorrel) == (1.0, 1.0, 1.0, 5.0, 500.0, 1.0)
    assert a.pe == pytest.approx(r.params.re * 0.71, rel=1e-12) and a.tref == 300.0
    assert r.thermal is not None and r.tparams is None


def test_clustered_cavity_cells():
    """The wall-clustered cavity: monotone nodes on the unit square, cell
    widths from (1 - beta)/n at the walls to (1 + beta)/n in the middle,
    the same in x and y."""
    n = 64
    case = deck.clustered_cavity(n, 1000.0, 1e-4, solver="rb_sor")
    x = case.x[:, 0]
    y = case.y[0, :]
    dx = np.diff(x)
    assert x[0] == 0.0 and abs(x[-1] - 1.0) < 1e-15
    assert np.all(dx > 0)
    assert abs(dx.min() * n - 0.5) < 0.01 and abs(dx.max() * n - 1.5) < 0.01
    assert np.allclose(x, y)
