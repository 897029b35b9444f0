"""Oracle geometry: Philox known answers, the sin/cos polynomial, BVH traversal
against brute force, and the watertight test against the reference's formulas."""
import numpy as np
import pytest

from helios_gb300 import scenes

# Published Random123 known-answer vectors for philox4x32-10.
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_kat(oracle_mod, ctr, key, out):
    assert tuple(int(x) for x in oracle_mod.philox(ctr, key)) == out


def test_sincos2pi_accuracy(oracle_mod):
    u = np.random.default_rng(0).random(200000).astype(np.float32)
    c, s = oracle_mod.sincos2pi(u)
    ref = 2 * np.pi * u.astype(np.float64)
    assert np.max(np.abs(c - np.cos(ref))) < 4e-7
    assert np.max(np.abs(s - np.sin(ref))) < 4e-7


def _mixed_scene(seed=1):
    a = scenes.homogeneous_canopy(n_leaves=3000, leaf=0.3, domain=5, seed=seed)
    b = scenes.orchard(nx=1, ny=1, leaves_per_tree=3000, side=0.3, seed=seed + 1)
    return (np.concatenate([a.T, b.T]), np.concatenate([a.ptype, b.ptype]), np.concatenate([a.twosided, b.twosided]))


def _rays(n, seed=0):
    rng = np.random.default_rng(seed)
    o = np.stack([rng.uniform(-1, 6, n), rng.uniform(-1, 6, n), rng.uniform(0, 6, n)], 1).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def test_bvh_equals_brute_force(oracle_mod):
    sc = oracle_mod.OracleScene(*_mixed_scene())
    o, d = _rays(100000)
    h0, t0, f0, cnt = sc.trace(o, d, mode=0)
    h1, t1, f1, _ = sc.trace(o, d, mode=1)
    assert np.array_equal(h0, h1)
    assert np.array_equal(t0[h0 >= 0], t1[h1 >= 0])
    assert np.array_equal(f0, f1)
    assert (h0 >= 0).mean() > 0.2
    assert cnt[0] / o.shape[0] < 200  # node visits per ray stay logarithmic-ish


def test_anyhit_agrees_with_closest(oracle_mod):
    sc = oracle_mod.OracleScene(*_mixed_scene(3))
    o, d = _rays(50000, 3)
    h0, *_ = sc.trace(o, d, mode=0)
    h3, *_ = sc.trace(o, d, mode=3)
    assert np.array_equal(h0 >= 0, h3 >= 0)


def test_watertight_vs_reference_formula(oracle_mod):
    """Hit IDs of the watertight test vs. the reference's patch/Shirley formulas
    (OptiX8DeviceCode.cu:369-489): identical except for counted grazing cases."""
    sc = oracle_mod.OracleScene(*_mixed_scene(5))
    o, d = _rays(100000, 5)
    h1, t1, f1, _ = sc.trace(o, d, mode=1)
    h2, t2, f2, _ = sc.trace(o, d, mode=2)
    differ = h1 != h2
    assert differ.mean() < 1e-3, differ.sum()
    same = (~differ) & (h1 >= 0)
    assert np.array_equal(f1[same], f2[same])
    np.testing.assert_allclose(t1[same], t2[same], rtol=1e-4, atol=1e-5)


def test_face_convention(oracle_mod):
    """A ray travelling against the normal meets the top face (face 1)."""
    T = scenes.helios_patch_T((0, 0, 0), (1, 1))[None]
    sc = oracle_mod.OracleScene(T, [0], [1])
    o = np.array([[0, 0, 1], [0, 0, -1]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, 1]], np.float32)
    h, t, f, _ = sc.trace(o, d, mode=1)
    assert list(h) == [0, 0] and list(f) == [1, 0]
    tri = scenes.triangle_T([0, 0, 0], [1, 0, 0], [0, 1, 0])  # normal +z
    sc = oracle_mod.OracleScene(tri, [1], [1])
    h, t, f, _ = sc.trace(np.array([[0.2, 0.2, 1], [0.2, 0.2, -1]], np.float32), d, mode=1)
    assert list(h) == [0, 0] and list(f) == [1, 0]


def test_watertight_shared_edge(oracle_mod):
    """Rays aimed exactly at the shared edge of two triangles of a mesh never fall
    through the crack (the property the watertight test guarantees)."""
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float64)
    T = np.concatenate([scenes.triangle_T(v[0], v[1], v[2]), scenes.triangle_T(v[0], v[2], v[3])])
    sc = oracle_mod.OracleScene(T, [1, 1], [1, 1])
    s = np.linspace(0.001, 0.999, 4001, dtype=np.float32)
    o = np.stack([s, s, np.full_like(s, 1.0)], 1)
    d = np.tile(np.array([[0, 0, -1]], np.float32), (s.size, 1))
    h, *_ = sc.trace(o, d, mode=1)
    assert (h >= 0).all()


def test_bvh_deterministic(oracle_mod):
    args = _mixed_scene(7)
    c1, p1, n1 = oracle_mod.OracleScene(*args).bvh()
    c2, p2, n2 = oracle_mod.OracleScene(*args).bvh()
    assert np.array_equal(c1, c2) and np.array_equal(p1, p2) and np.array_equal(n1, n2)
    assert np.all(np.diff(c1.astype(np.float64)) >= 0)
    assert np.array_equal(np.sort(p1), np.arange(p1.size))
