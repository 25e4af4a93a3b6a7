"""Host geometry builder against the reference's mesh arrays, bit for bit."""
import numpy as np
import pytest

import _golden as G
from pyhype_gb300.mesh import RectagularMeshGenerator, build_block_geometry


@pytest.mark.parametrize("name", G.cases())
def test_block_geometry_bitwise(name):
    z = G.load(name)
    nx, ny = int(z["nx"]), int(z["ny"])
    for k, b in enumerate(z["blk_ids"]):
        c = z["corners"][k]
        g = build_block_geometry({"SW": list(c[0]), "SE": list(c[1]), "NW": list(c[2]), "NE": list(c[3])}, nx, ny)
        p = f"geo{int(b)}_"
        pairs = [("nodes_x", g.nodes_x), ("nodes_y", g.nodes_y), ("xc", g.xc), ("yc", g.yc),
                 ("A", g.A), ("dx", g.dx), ("dy", g.dy)]
        for s in "EWNS":
            L, th, nxx, nyy = g.side(s)
            pairs += [("L" + s, L), ("th" + s, th), ("nx" + s, nxx), ("ny" + s, nyy),
                      ("qx" + s, getattr(g, f"q{s}_x")), ("qy" + s, getattr(g, f"q{s}_y")),
                      # the rotations take cos/sin of theta per element at run time
                      ("cos_scalar" + s, np.cos(th)), ("sin_scalar" + s, np.sin(th))]
        for key, arr in pairs:
            assert np.array_equal(arr, z[p + key]), f"block {b} {key}"
        assert g.is_cartesian == bool(z[p + "is_cartesian"])


def test_rectangular_generator_corners():
    z = G.load("m2x4_40")
    m = RectagularMeshGenerator.generate(["Reflection"], ["Reflection"], ["Reflection"], ["Reflection"],
                                         10.0, 0.0, 20.0, 0.0, 2, 4)
    cs = np.array([[m.dict[b][k] for k in ("SW", "SE", "NW", "NE")] for b in sorted(m.dict)])
    assert np.array_equal(cs, z["corners"])
    nbr = np.array([[-1 if m.dict[b]["Neighbor" + s] is None else m.dict[b]["Neighbor" + s] for s in "EWNS"]
                    for b in sorted(m.dict)])
    assert np.array_equal(nbr, z["neighbors"])
