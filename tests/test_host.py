"""Host-side logic: drand48 / gaussian stream, input keys and constructor
defaults per model, and the configuration file format."""
import ctypes
import math
import os

import numpy as np
import pytest

from rheocell_gb300 import abi, generator as g, host


def test_drand48_matches_libc():
    libc = ctypes.CDLL(None)
    libc.drand48.restype = ctypes.c_double
    for seed in (1, 4982, 123456789, -5):
        libc.srand48(ctypes.c_long(seed))
        r = host.Drand48(seed)
        for _ in range(200):
            assert r.drand48() == libc.drand48()


def test_gaussian_pairs_and_cache():
    r = host.Drand48(7)
    a = r.gaussian()
    assert r.has_cached == 1
    b = r.gaussian()
    assert r.has_cached == 0 and b == r.cached and a != b


def test_params_defaults_per_model():
    base = dict(R=8, dt=0.1, zetaQ_self=0.1, zetaQ_inter=0, J_Q=0, friction=1, friction_cell=0, beta=0)
    p = host.make_params(dict(base, interaction_type="simplefield", **{"lambda": 2.0}))
    assert p.lambda_ == 2.5, "SimpleMultiField::get_settings does not read lambda"
    p = host.make_params(dict(base, interaction_type="activenematic", friction=3))
    assert list(p.friction) == [3.0, 3.0] and list(p.zetaQ_self) == [0.0, 0.1]
    p = host.make_params(dict(base, interaction_type="wetpolarmodel", friction=2, friction_cell=1))
    assert list(p.friction) == [1.0, 2.0] and list(p.friction_cell) == [0.0, 1.0]
    assert p.cg_restart_every == 10 and p.cg_tolerance == 1e-4
    p = host.make_params(dict(base, interaction_type="wetmodel", CGtolerance=1e-8))
    assert p.cg_restart_every == 100 and p.cg_tolerance == 1e-8 and p.gamma == 0.01


def test_params_reject_unprovided():
    base = dict(R=8, dt=0.1, zetaQ_self=0, zetaQ_inter=0, J_Q=0, friction=1, friction_cell=0, beta=0,
                interaction_type="wetpolarmodel")
    with pytest.raises(ValueError):
        host.make_params(dict(base, interaction_type="lebcwetmodel"))
    with pytest.raises(ValueError):
        host.make_params(dict(base, box="channel"))
    with pytest.raises(ValueError):
        host.make_params(dict(base, box="orthogonal", type="channel_walls"))
    with pytest.raises(ValueError):
        host.box_walls(dict(base, type="square_walls"), 64)  # lambda_wall is required
    with pytest.raises(ValueError):
        host.make_params({k: v for k, v in base.items() if k != "friction_cell"})


def test_wall_masks():
    # SquareWalls: x < lambda-1 or x > L-lambda, y < lambda or y > L-lambda
    w = host.box_walls(dict(type="square_walls", lambda_wall=3), 16).reshape(16, 16)
    assert w[:, 0].all() and w[:, 1].all() and not w[5, 2] and w[5, 14] and not w[5, 13]
    assert w[0].all() and w[2].all() and not w[3, 5] and w[14, 5] and not w[13, 5]
    # CircleWalls: centre open, corners closed; TriangleWalls: a closed border
    c = host.box_walls(dict(type="circle_walls", lambda_wall=2), 32).reshape(32, 32)
    assert c[0, 0] == 1 and c[16, 16] == 0 and c[16, 1] == 1
    t = host.box_walls(dict(type="triangle_walls", lambda_wall=4), 64).reshape(64, 64)
    assert t[0].all() and t[:, 0].all() and not t[32, 32]
    # no walls: None; wall_slip <= 0 on the periodic box closes every site
    assert host.box_walls({}, 8) is None
    assert not host.box_walls(dict(wall_slip=0), 8).any()


def test_nemq_seeding_order():
    m = g.make_monolayer(64, 4, seed=1)
    keys = dict(interaction_type="wetmodel", seed="5")
    cells, rng = host.make_cells(m, keys, 5)
    r = host.Drand48(5)
    for i in range(4):
        th = float(np.float32(math.pi)) * (1 - 2 * r.drand48())
        q0 = math.cos(2 * th)
        assert cells.arr[i].nemq_x == math.sqrt((1 + q0 / math.hypot(q0, math.sin(2 * th))) / 2)
    polar = dict(keys, interaction_type="wetpolarmodel")
    _, rng2 = host.make_cells(m, polar, 5)
    assert rng2.state != rng.state  # read_topology draws once per cell first


def test_conf_roundtrip(tmp_path):
    m = g.make_monolayer(64, 4, seed=2)
    p = tmp_path / "c.dat"
    g.write_conf(str(p), m)
    m2 = g.read_conf(str(p))
    assert m2.L == 64 and m2.n == 4
    for a, b in zip(m.cells, m2.cells):
        assert (a.lx, a.ly, a.corner, a.offset) == (b.lx, b.ly, b.corner, b.offset)
        np.testing.assert_array_equal(a.box_index, b.box_index)
        np.testing.assert_allclose(a.phi, b.phi, rtol=1e-14, atol=1e-300)
    g.write_conf(str(p) + "2", m2)
    assert open(str(p)).read() == open(str(p) + "2").read()


def test_generator_shapes():
    m = g.make_monolayer(140, 100, seed=1)
    assert m.sites == 100 * 41 * 41
    assert all(c.lx == 41 and 0 <= c.com[0] < 140 for c in m.cells)
    phi = np.concatenate([c.phi for c in m.cells])
    assert phi.max() < 1.0 and phi.min() > 0.0


def test_read_input(tmp_path):
    p = tmp_path / "input"
    p.write_text("a = 1 # c\n# full\nb=  x y \n a = 2\n")
    k = host.read_input(str(p), {"c": 3})
    assert k == {"a": "2", "b": "x y", "c": "3"}


def test_bench_workloads_start_within_the_overlap_limit():
    """Every bench workload's initial condition keeps at most 20 patches on a
    box site: the wet models abort beyond that (store_max_size,
    WetModel.cpp:58, :475-480), and the 123 % area fraction of the wet
    configurations is well inside it (mean coverage n P^2 / L^2 = 10.26)."""
    import bench
    from rheocell_gb300 import generator as gen

    def coverage(m):
        L = m.L
        cnt = np.zeros(L * L, np.int64)
        for c in m.cells:
            cx, cy = c.corner % L, c.corner // L
            idx = (((cy + np.arange(c.ly)) % L)[:, None] * L + ((cx + np.arange(c.lx)) % L)[None, :]).ravel()
            cnt += np.bincount(idx, minlength=L * L)
        return cnt

    for L, n in ((140, 100), (256, 400), (512, 1600), (1024, 6400)):
        cnt = coverage(gen.make_monolayer(L, n, seed=1))
        assert cnt.max() <= 20
        assert cnt.sum() == n * 41 * 41
    for L, n, seed in bench.ensemble_members():
        assert coverage(gen.make_monolayer(L, n, seed=seed)).max() <= 20
