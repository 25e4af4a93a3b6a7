"""The benchmark configurations are the ones the workloads name: the 512-instance
explosion ensemble's distributions, the double-Mach reflection's domain, blocks,
states and scheme, the multiblock explosion's layout and scheme, and the adjoint
problem.  Host-side only (no GPU)."""
import numpy as np
import pytest

from pyhype_gb300.batch import BASE_P, BASE_RHO, explosion_ensemble


def test_explosion_ensemble_distributions():
    inst = explosion_ensemble(512, seed=0)
    assert len(inst) == 512
    sizes = set(range(64, 513, 32))
    nx = np.array([i.nx for i in inst])
    ny = np.array([i.ny for i in inst])
    assert set(nx) <= sizes and set(ny) <= sizes
    assert len(set(nx)) == len(sizes) and len(set(ny)) == len(sizes)  # every size drawn
    for i in inst:
        assert i.lx == i.nx / 10 and i.ly == i.ny / 10
        assert 0.1 <= i.half_width / min(i.lx, i.ly) <= 0.3
        assert i.half_width <= i.cx <= i.lx - i.half_width and i.half_width <= i.cy <= i.ly - i.half_width
        assert 2.0 <= i.p_ratio <= 20.0 and i.rho_ratio == 4.0
    lr = np.log([i.p_ratio for i in inst])
    assert abs(lr.mean() - 0.5 * (np.log(2) + np.log(20))) < 0.1  # log-uniform
    again = explosion_ensemble(512, seed=0)
    assert [(a.nx, a.ny, a.cx, a.p_ratio) for a in inst] == [(b.nx, b.ny, b.cx, b.p_ratio) for b in again]
    assert (BASE_RHO, BASE_P) == (1.1742, 101100.0)


def test_double_mach_configuration():
    from pyhype_gb300.configs import DMR_POST, DMR_PRE, double_mach
    from pyhype_gb300.states import PrimitiveState

    cfg, gen = double_mach()
    assert (cfg.nx, cfg.ny) == (400, 500)
    assert cfg.fvm_flux_function_type == "HLLL" and cfg.fvm_slope_limiter_type == "Venkatakrishnan"
    assert cfg.fvm_gradient_type == "GreenGauss" and cfg.reconstruction_type is PrimitiveState
    assert cfg.time_integrator == "SSPRK2" and cfg.CFL == 0.4 and cfg.t_final == 0.2
    d = gen.dict
    assert len(d) == 5
    xs = sorted(x for b in d.values() for x in (b["SW"][0], b["SE"][0]))
    ys = sorted(y for b in d.values() for y in (b["SW"][1], b["NW"][1]))
    assert (xs[0], xs[-1], ys[0], ys[-1]) == (0.0, 4.0, 0.0, 1.0)
    widths = [b["SE"][0] - b["SW"][0] for b in d.values()]
    assert np.allclose(widths, 0.8)                     # 400 cells of 0.002 per block
    assert DMR_PRE == [1.4, 0.0, 0.0, 1.0]
    assert np.allclose(DMR_POST, [8.0, 8.25 * np.cos(np.pi / 6), -8.25 * np.sin(np.pi / 6), 116.5])


def test_multiblock_explosion_configuration():
    from pyhype_gb300.configs import explosion_multiblock
    from pyhype_gb300.states import ConservativeState

    cfg, mesh = explosion_multiblock(1024)
    assert (cfg.nx, cfg.ny) == (1024, 1024)
    assert cfg.fvm_flux_function_type == "Roe" and cfg.fvm_slope_limiter_type == "Venkatakrishnan"
    assert cfg.time_integrator == "RK4" and cfg.CFL == 0.8 and cfg.t_final == 0.07
    assert cfg.reconstruction_type is ConservativeState
    d = mesh.dict
    assert len(d) == 8
    xs = [x for b in d.values() for x in (b["SW"][0], b["NE"][0])]
    ys = [y for b in d.values() for y in (b["SW"][1], b["NE"][1])]
    assert (min(xs), max(xs), min(ys), max(ys)) == (0.0, 10.0, 0.0, 20.0)


def test_adjoint_problem_configuration():
    torch = pytest.importorskip("torch")
    from pyhype_gb300.adjoint import adjoint_problem, smoothed_explosion

    P = adjoint_problem(n=256)
    assert P.nblocks == 1 and (P.blocks[0].nx, P.blocks[0].ny) == (256, 256)
    g = P.block_geometry[0]
    assert g.nodes_x.min() == 0.0 and g.nodes_x.max() == 10.0 and g.nodes_y.max() == 10.0
    U = smoothed_explosion(P, 4.0, 2.0, 5.0, device="cpu")
    assert U.shape == (4, 256 * 256) and U.dtype == torch.float64 and bool(torch.isfinite(U).all())
