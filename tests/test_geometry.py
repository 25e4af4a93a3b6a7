"""Host geometry builder against the reference's mesh arrays, bit for bit."""
import numpy as np
import pytest

import _golden as G
from pyhype_gb300.mesh import RectagularMeshGenerator, build_block_geometry
from pyhype_gb300.mesh.quad_mesh import quadrature_points


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
        nqp = int(z["nqp"]) if "nqp" in z.files else 1
        qps = quadrature_points(g, nqp)
        for s in "EWNS":
            L, th, nxx, nyy = g.side(s)
            pairs += [("L" + s, L), ("th" + s, th), ("nx" + s, nxx), ("ny" + s, nyy),
                      # the rotations take cos/sin of theta per element at run time
                      ("cos_scalar" + s, np.cos(th)), ("sin_scalar" + s, np.sin(th))]
            if nqp == 1:
                pairs += [("qx" + s, getattr(g, f"q{s}_x")), ("qy" + s, getattr(g, f"q{s}_y"))]
            else:  # every point of the multi-point rule
                for k, (_, pts) in enumerate(qps):
                    pairs += [(f"qx{s}_{k}", pts[s][0]), (f"qy{s}_{k}", pts[s][1])]
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


@pytest.mark.parametrize("name", ["m2x4_40", "dmr_example", "p100"])
def test_problem_planes_from_own_geometry_equal_reference_geometry(name):
    """On this platform the geometry planes built from the product's own mesh code are
    the ones built from the reference's recorded arrays."""
    z = G.load(name)
    a = G.problem(z, reference_geometry=True)
    b = G.problem(z, reference_geometry=False)
    import ctypes
    import numpy as np
    for k in range(12):
        pa = np.ctypeslib.as_array(a.geometry.cell[k], shape=(a.ncell,))
        pb = np.ctypeslib.as_array(b.geometry.cell[k], shape=(b.ncell,))
        assert np.array_equal(pa, pb), k
    for k in range(5):
        assert np.array_equal(np.ctypeslib.as_array(a.geometry.vface[k], shape=(a.nvface,)),
                              np.ctypeslib.as_array(b.geometry.vface[k], shape=(b.nvface,)))
        assert np.array_equal(np.ctypeslib.as_array(a.geometry.hface[k], shape=(a.nhface,)),
                              np.ctypeslib.as_array(b.geometry.hface[k], shape=(b.nhface,)))
