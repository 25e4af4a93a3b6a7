"""The CPU oracle against fixtures produced by the pyHype reference itself.

Bit-exact (value equality; -0.0 == +0.0): every per-operator intermediate of one
residual evaluation, the dt of every step, and the state after every step (through
per-step fingerprints plus full snapshots)."""
import numpy as np
import pytest

import _golden as G
from oracle.oracle import Oracle

CASES = G.cases()
OPS_CASES = [c for c in CASES if "ops_state" in G.load(c).files]


@pytest.mark.parametrize("name", OPS_CASES)
def test_operator_intermediates(name):
    z = G.load(name)
    P = G.problem(z)
    t = float(z["ops_t"]) if "ops_t" in z.files else 0.0
    dudt, dbg = Oracle(P).residual(P.to_soa(list(z["ops_state"])), t=t, debug=True)
    for b in range(P.nblocks):
        p = f"ops{int(z['blk_ids'][b])}_"
        vf = P.vface_block(dbg["vflux"], b)
        hf = P.hface_block(dbg["hflux"], b)
        pairs = {
            "gx": (P.from_soa(dbg["gx"])[b], z[p + "gx"]),
            "gy": (P.from_soa(dbg["gy"])[b], z[p + "gy"]),
            "phi": (P.from_soa(dbg["phi"])[b], z[p + "phi"]),
            "xL": (P.vface_block(dbg["vL"], b), z[p + "xL"]),
            "xR": (P.vface_block(dbg["vR"], b), z[p + "xR"]),
            "yL": (P.hface_block(dbg["hL"], b).transpose(1, 0, 2), z[p + "yL"]),
            "yR": (P.hface_block(dbg["hR"], b).transpose(1, 0, 2), z[p + "yR"]),
            "xF": (P.vface_block(dbg["vflux_raw"], b), z[p + "xF"]),
            "yF": (P.hface_block(dbg["hflux_raw"], b).transpose(1, 0, 2), z[p + "yF"]),
            "fluxE": (vf[:, 1:], z[p + "fluxE"]),
            "fluxW": (vf[:, :-1], z[p + "fluxW"]),
            "fluxN": (hf[1:], z[p + "fluxN"]),
            "fluxS": (hf[:-1], z[p + "fluxS"]),
            "dUdt": (P.from_soa(dudt)[b], z[p + "dUdt"]),
        }
        for key, (mine, ref) in pairs.items():
            assert mine.shape == ref.shape, (key, mine.shape, ref.shape)
            assert np.array_equal(mine, ref), f"block {b} {key}: max diff {np.max(np.abs(mine - ref))}"


def ghost_pairs(P, z, layer):
    """(mine, reference) ghost arrays per block side; the reference records the
    reconstruction block's ghosts as (ny, 1, 4) / (1, nx, 4)."""
    for b, sides in enumerate(P.split_ghosts(layer)):
        p = f"ops{int(z['blk_ids'][b])}_"
        for side, mine in sides.items():
            yield f"block {b} ghost{side}", mine, z[p + "ghost" + side].reshape(-1, 4)


@pytest.mark.parametrize("name", OPS_CASES)
def test_ghost_layer(name):
    """Halo fill + boundary conditions + conversion to the reconstruction variables."""
    z = G.load(name)
    P = G.problem(z)
    t = float(z["ops_t"]) if "ops_t" in z.files else 0.0
    layer = Oracle(P).ghost_layer(P.to_soa(list(z["ops_state"])), t=t)
    for key, mine, ref in ghost_pairs(P, z, layer):
        assert mine.shape == ref.shape, key
        assert np.array_equal(mine, ref), f"{key}: max diff {np.max(np.abs(mine - ref))}"


@pytest.mark.parametrize("name", CASES)
def test_steps_bitwise(name):
    z = G.load(name)
    P = G.problem(z)
    O = Oracle(P)
    U = P.to_soa(list(z["ic"]))
    tab = z["tableau"]
    t, tf = 0.0, G.t_final(z)
    for step in range(1, int(z["steps"]) + 1):
        dt = float(O.dt(U)[0])
        if tf - t < dt:
            dt = tf - t
        assert dt == z["dts"][step - 1], f"step {step}: dt {dt!r} != {z['dts'][step - 1]!r}"
        U = O.step(U, tab, dt, t)
        t += dt
        assert t == z["ts"][step - 1]
        blocks = P.from_soa(U)
        if f"state_{step}" in z.files:
            assert np.array_equal(np.stack(blocks), z[f"state_{step}"]), f"state after step {step}"
        assert G.fingerprint(blocks) == str(z["fingerprints"][step - 1]), f"fingerprint after step {step}"
    assert O.realizable(U).ok == 1
