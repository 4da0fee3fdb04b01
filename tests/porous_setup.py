"""Porous-region layouts (porous_region keyword, PorRegCnst constants) for
the porous momentum terms: PorosCoef and the porosity division of the
convective coefficients (src/momentum.f:296-324, 621-649, 1115-1226)."""
import numpy as np

from wolfd2_gb300 import deck

LAYOUTS = {
    # porous regions 2 and 3 share the border i = 24 (divided twice there)
    "row": ("number_of_regions 3 1\n i_borders 12 24\n j_borders\n"
            "porous_region 2 1 carman-kozeny 0.6 0.05 0.5\n"
            "porous_region 3 1 kaviany 0.45 0.08 0.3\n"
            "inlet 1 1 west nv 1.0\n outlet 3 1 east fd\n", 40, 16),
    # three porous regions of four around a non-porous one: shared borders
    # in i and in j, PorosCoef's last writer changing along them
    "quad": ("number_of_regions 2 2\n i_borders 18\n j_borders 9\n"
             "porous_region 1 1 carman-kozeny 0.7 0.04 0.4\n"
             "porous_region 2 1 happen-brenner 0.5 0.06 0.6\n"
             "porous_region 2 2 carman-kozeny 0.55 0.05 0.2\n"
             "inlet 1 1 west nv 1.0\n inlet 1 2 west nv 1.0\n"
             "outlet 2 1 east mc\n outlet 2 2 east mc\n", 36, 18),
}


# a lid-driven cavity on a curvilinear grid with two porous regions stacked
# in j (their shared border divided twice by the Y loop), non-Cartesian Ppe
CURVI = ("number_of_regions 3 2\n i_borders 13 25\n j_borders 11\n"
         "wall 1 2 north tv 1.0\n wall 2 2 north tv 1.0\n wall 3 2 north tv 1.0\n"
         "porous_region 2 1 carman-kozeny 0.6 0.05 0.5\n"
         "porous_region 2 2 kaviany 0.5 0.06 0.4\n")


def case(name: str):
    if name == "curvi":
        c = deck.cavity(36, 200.0, 0.004, solver="rb_sor", ny=24)
        c.regions = deck.parse_bc_section(CURVI, c.nx, c.ny, re=c.params.re)
        c.bc_text = CURVI
        X, Y = c.x.copy(), c.y.copy()
        c.x = X + 0.02 * np.sin(np.pi * X) * np.sin(np.pi * Y)
        c.y = Y + 0.015 * np.sin(2 * np.pi * X) * np.sin(np.pi * Y)
        c.params.lcartes = 0
        return c
    text, nx, ny = LAYOUTS[name]
    c = deck.channel(nx, ny, 300.0, 0.003, length=2.0, solver="rb_sor")
    c.regions = deck.parse_bc_section(text, c.nx, c.ny, re=c.params.re)
    c.bc_text = text
    return c
