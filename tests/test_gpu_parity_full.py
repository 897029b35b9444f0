"""GPU parity at the benchmarked sizes, against the FP64 oracle on the same Philox ray set.

- the plain canopy at its stated size: 20,001 primitives, 100 direct / 300 (18^2 = 324)
  diffuse rays, depth 3, sun + sky, seed 0 (53.8 M rays);
- the 1 M-triangle orchard of the headline benchmark, all three bands (PAR, NIR, longwave
  emission), depth 5, at reduced ray counts (9 direct, 16 diffuse: 201 M rays) so the
  oracle finishes in seconds on the host cores -- the kernels, tree and scene are the
  benchmark's own;
- the device LBVH against the host build at 1 M primitives: Morton codes, the radix-sort
  permutation (ties included), Karras topology and refit boxes, bit for bit.
"""
import numpy as np
import pytest

from helios_gb300 import workloads

from helpers import run_oracle

pytestmark = pytest.mark.gpu

FLUX_RTOL = 1e-4  # per-primitive relative flux error vs the FP64 oracle


@pytest.fixture(scope="module")
def orchard_1m():
    rad, sc = workloads.orchard_model(direct_rays=9, diffuse_rays=16, depth=5)
    rad.updateGeometry()
    return rad, sc


def test_canopy_full_size_vs_oracle(oracle_mod):
    rad, sc = workloads.canopy_model()
    assert sc.n == 20001
    rad.setSeed(0)
    got = rad.runBand("SW")
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=0)
    err = workloads.max_rel_err(got, ref)
    print(f"canopy {sc.n} primitives, {st['rays']} rays: max rel err {err:.3e}")
    assert err <= FLUX_RTOL, err
    assert rad.last_stats["rays"] == st["rays"]
    assert st["rays"] > 50_000_000


def test_orchard_1m_three_bands_vs_oracle(oracle_mod, orchard_1m):
    rad, sc = orchard_1m
    assert sc.n == 1_000_000
    rad.setSeed(3)
    got = rad.runBand(workloads.ORCHARD_BANDS)
    ref, st = run_oracle(rad, workloads.ORCHARD_BANDS, oracle_mod, seed=3)
    assert got.shape == ref.shape == (sc.n, 3)
    errs = [workloads.max_rel_err(got[:, b], ref[:, b]) for b in range(3)]
    print(f"orchard {sc.n} triangles, {st['rays']} rays: max rel err per band {errs}")
    assert max(errs) <= FLUX_RTOL, errs
    assert rad.last_stats["rays"] == st["rays"]


def test_bvh_bit_exact_1m(oracle_mod, orchard_1m):
    rad, sc = orchard_1m
    T, ty, ts = rad.geometry_arrays()
    c1, p1, n1 = rad.ctx.bvh()
    c2, p2, n2 = oracle_mod.OracleScene(T, ty, ts).bvh()
    assert c1.shape[0] == 1_000_000
    assert np.array_equal(c1, c2)
    assert np.array_equal(p1, p2)
    assert np.array_equal(n1[:, 12:14], n2[:, 12:14])
    assert np.array_equal(n1[:, :12].view(np.float32), n2[:, :12].view(np.float32))
