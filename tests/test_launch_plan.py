"""Launch planning on the host (hrt_plan_launch_chunks): ray ids inside one trace launch are
32-bit, so passes of 2^31 rays or more run as consecutive launches over primitive chunks.

Pure host arithmetic in libhrt.so; runs without a GPU."""
import pytest

from helios_gb300 import _hrt

LIMIT = 1 << 31


@pytest.fixture(scope="module")
def lib(hrt_lib):
    return hrt_lib


@pytest.mark.parametrize("count,rays", [
    (1_000_000, 225 * 2),          # orchard diffuse pass, both faces: one launch
    (1_000_000, 5041 * 2),         # setDiffuseRayCount(5000) on 1 M primitives: 10.1 G rays
    (4_000_000, 400 * 2),          # deep-scatter scene, 20 x 20 rays, both faces
    (20_001, 100),                 # canopy direct pass
    (2**32 - 1, 1),                # the largest primitive count, one ray each
    (2**32 - 1, 3),
    (7, 2**31),                    # one primitive's rays fill a launch
    (1, 1),
])
def test_chunks_cover_every_primitive_below_the_limit(lib, count, rays):
    k, per = _hrt.plan_launch_chunks(count, rays)
    assert per >= 1
    assert per * rays <= LIMIT            # no launch reaches 2^31 ray ids
    assert k * per >= count               # every primitive is in some launch
    assert (k - 1) * per < count          # and no launch is empty
    if count * rays < LIMIT:
        assert k == 1


def test_verdict_example_splits(lib):
    k, per = _hrt.plan_launch_chunks(1_000_000, 5041 * 2)
    assert k == 5 and per == LIMIT // (5041 * 2)


def test_lowered_limit(lib):
    k, per = _hrt.plan_launch_chunks(2001, 100, 30_000)
    assert per == 300 and k == 7
    # limits above 2^31 are clamped to it
    k2, per2 = _hrt.plan_launch_chunks(10**9, 1000, 1 << 40)
    assert per2 == LIMIT // 1000 and k2 == -(-10**9 // per2)


def test_empty_and_oversized(lib):
    assert _hrt.plan_launch_chunks(0, 100) == (0, LIMIT // 100)
    with pytest.raises(_hrt.HrtError) as e:
        _hrt.plan_launch_chunks(10, LIMIT + 1)
    assert e.value.code == _hrt.HRT_EUNSUPPORTED
    with pytest.raises(_hrt.HrtError):
        _hrt.plan_launch_chunks(10, 50, 49)
