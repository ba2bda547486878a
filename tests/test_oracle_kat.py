"""Known-answer tests of the FP64 oracle (CPU only).

The reference ships no tests or golden vectors; these KATs pin the oracle's kernels and
integer bookkeeping on hand-computable cases, written from the formulas of
src/MPS_Computer/MPSSPHKernel.cuh:28-84 (poly6 / spiky / cubic spline / surface tension) and the
neighbour rules of src/MPS_Object/MPSSpatialHash.cuh:147-271.
"""
import math

import numpy as np
import pytest

PI = math.pi


def w_poly6(q, h):
    return 315.0 / (64.0 * PI) / h ** 3 * (1 - q * q) ** 3 if q < 1 else 0.0


def g_spiky(q, h):  # scalar G with grad W = G * x_ij
    d = q * h
    return -45.0 / PI / d * ((1 - q) / h ** 2) ** 2 if 1e-20 <= q < 1 else 0.0


def w_cubic(q, h):
    if q >= 1:
        return 0.0
    if q >= 0.5:
        return 8.0 / PI * 2.0 * ((1 - q) / h) ** 3
    return 8.0 / PI / h ** 3 * ((6 * q - 6) * q * q + 1)


def g_cubic(q, h):
    d = q * h
    if q < 1e-20 or q >= 1:
        return 0.0
    if q > 0.5:
        return -48.0 / PI / d * ((1 - q) / h ** 2) ** 2
    return 48.0 / PI / d / h ** 4 * (3 * q - 2) * q


def _two_particle(orc, q, cubic):
    r = 0.1
    h = 4 * r
    mat = dict(radius=h, mass=1.0, density=1.0, volume=0.5, viscosity=0.0, xsph=0.0, surface_tension=0.0)
    phys = dict(dt=0.01, gravity=(0, 0, 0), min=(-5, -5, -5), max=(5, 5, 5))
    o = orc.Oracle(orc.params(mat, phys, dict(kernel=cubic), hash_cell=h))
    pos = np.array([[0.0, 0.0, 0.0], [q * h, 0.0, 0.0]])
    o.set_boundary(np.zeros((0, 3)), np.zeros(0))
    o.set_fluid(pos, np.zeros((2, 3)), np.ones(2), np.full(2, r))
    for ph in (orc.NEIGHBORS, orc.DENSITY, orc.ALPHA):
        o.phase(ph)
    return o, h, mat["volume"]


@pytest.mark.parametrize("cubic", [0, 1])
@pytest.mark.parametrize("q", [0.0, 0.25, 0.5, 0.99, 1.0])
def test_two_particle_density_and_alpha(orc, q, cubic):
    o, h, V = _two_particle(orc, q, cubic)
    W = w_cubic if cubic else w_poly6
    G = g_cubic if cubic else g_spiky
    linked = q < 1.0
    rho = o.get("density")
    expect = V * (W(0.0, h) + (W(q, h) if linked else 0.0))
    assert rho[0] == pytest.approx(expect, rel=1e-13)
    assert rho[1] == pytest.approx(expect, rel=1e-13)
    # alpha = 1 / (|V G x|^2 + |V G x|^2) for one neighbour; 0 below the 1e-20 clamp
    g = V * G(q, h) * (q * h) if linked else 0.0
    f = 2 * g * g
    alpha = o.get("alpha")
    if f > 1e-20:
        assert alpha[0] == pytest.approx(1.0 / f, rel=1e-12)
    else:
        assert alpha[0] == 0.0


def test_lattice_center_has_26_neighbours(orc):
    s = 0.1
    r = s / 2  # h = 4 r = 2 s > sqrt(3) s
    pts = np.array([[x, y, z] for z in range(3) for y in range(3) for x in range(3)], float) * s
    mat = dict(radius=4 * r, mass=1.0, density=1.0, volume=s ** 3, viscosity=0, xsph=0, surface_tension=0)
    phys = dict(dt=0.01, gravity=(0, 0, 0), min=(-1, -1, -1), max=(1, 1, 1))
    o = orc.Oracle(orc.params(mat, phys, hash_cell=4 * r))
    o.set_boundary(np.zeros((0, 3)), np.zeros(0))
    o.set_fluid(pts, np.zeros_like(pts), np.ones(27), np.full(27, r))
    o.phase(orc.NEIGHBORS)
    idx = o.get("nei_ff_idx")
    counts = np.diff(idx)
    assert counts[13] == 26
    # a corner sees its 7 cube neighbours plus the 3 at distance 2 s < 2 s? (no: strict <) -> 7
    assert counts[0] == 7


def test_new_scheme_keys_sort_ranges(orc):
    g = orc.grid((0.0, 0.0, 0.0), 1.0, (4, 3, 2))
    pts = np.array([[0.5, 0.5, 0.5], [3.5, 2.5, 1.5], [1.2, 0.1, 0.9], [0.7, 0.2, 0.3], [-3.0, 9.0, 0.5],
                    [1.9, 0.9, 0.1], [3.99, 0.0, 1.0], [np.nan, 0.5, 0.5]], np.float32)
    p4 = np.zeros((8, 4), np.float32)
    p4[:, :3] = pts
    keys = orc.new_keys(p4, g)
    # columns of 2 x 2 rows (y, z) along x: col = (cz // 2) * ceil(ny / 2) + cy // 2,
    # key = ((col * nx + cx) * 2 + cz % 2) * 2 + cy % 2, with clamping; NaN -> cell 0 on that axis.
    # cells: (0,0,0) (3,2,1) (1,0,0) (0,0,0) (0,2,0) (1,0,0) (3,0,1) (0,0,0); ceil(3 / 2) = 2
    expect = [0, ((1 * 4 + 3) * 2 + 1) * 2 + 0, ((0 * 4 + 1) * 2 + 0) * 2 + 0, 0, ((1 * 4 + 0) * 2 + 0) * 2 + 0,
              ((0 * 4 + 1) * 2 + 0) * 2 + 0, ((0 * 4 + 3) * 2 + 1) * 2 + 0, 0]
    assert expect == [0, 30, 4, 0, 16, 4, 14, 0]
    assert keys.tolist() == expect
    sk, sv = orc.new_stable_sort(keys, np.arange(8, dtype=np.uint32))
    assert sv.tolist() == [0, 3, 7, 2, 5, 6, 4, 1]  # ties keep input order
    cells, st, en = orc.new_cell_ranges(sk)
    assert cells.tolist() == [0, 4, 14, 16, 30]
    assert st.tolist() == [0, 3, 5, 6, 7]
    assert en.tolist() == [3, 5, 6, 7, 8]


def test_fp32_counts_match_fp64_reference_counts(orc, mps):
    from mps_cuda_gb300 import scenes
    sc = scenes.dam_break_small(8, seed=3)
    o = orc.from_scene(sc)
    o.phase(orc.NEIGHBORS)
    ref_ff = np.diff(o.get("nei_ff_idx"))
    ref_fb = np.diff(o.get("nei_fb_idx"))
    h = 4 * sc.pos4[0, 3]
    lo = np.asarray(sc.physics["min"]) - h
    dims = [int(np.ceil((sc.physics["max"][a] - sc.physics["min"][a]) / h)) + 2 for a in range(3)]
    g = orc.grid(tuple(np.float32(lo)), np.float32(h), dims)
    q4 = sc.pos4.copy()
    q4[:, 3] *= 4
    b4 = sc.bpos4.copy()
    b4[:, 3] *= 4
    kq = orc.new_keys(q4, g)
    kq_s, order = orc.new_stable_sort(kq, np.arange(sc.n, dtype=np.uint32))
    kb = orc.new_keys(b4, g)
    kb_s, border = orc.new_stable_sort(kb, np.arange(sc.nb, dtype=np.uint32))
    cf = orc.new_nbr_counts(q4[order], q4[order], kq_s, g, True)
    cb = orc.new_nbr_counts(q4[order], b4[border], kb_s, g, False)
    # FP32 and FP64 tests agree except for pairs within 1e-6 h of the support radius
    assert np.abs(cf.astype(int) - ref_ff[order].astype(int)).max() <= 1
    assert (cf != ref_ff[order]).mean() < 1e-3
    assert (cb != ref_fb[order]).mean() < 1e-3


def test_oracle_deterministic_across_threads(orc, mps):
    from mps_cuda_gb300 import scenes
    sc = scenes.dam_break_small(8, seed=1)
    outs = []
    for t in (1, 4):
        o = orc.from_scene(sc, threads=t)
        o.step(2)
        outs.append((o.get("pos"), o.get("vel"), o.get("density")))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
