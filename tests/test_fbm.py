"""fBm generator (the out-of-core workload's input) on the host: the
library's generator, which a data-source callback runs per brick, against
the oracle's independent restatement, byte for byte. Parity unpinned (no
reference test covers this synthetic input)."""
import numpy as np
import pytest


@pytest.mark.parametrize("dtype,voxels,block,seed,octaves", [
    (2, 256, 32, 1234, 6), (1, (96, 64, 80), 16, 7, 3), (2, (130, 70, 40), 16, 99, 1)])
def test_host_fbm_matches_oracle(native, oracle, dtype, voxels, block, seed, octaves):
    import livre_gb300 as lv
    vi = lv.VolumeInformation(voxels, block, 1, dtype=dtype)
    ovol = oracle.volume(voxels, block, 1)
    fp = oracle.fbm_params(seed, octaves, 2.0, 0.5, 8.0, dtype=dtype)
    nodes = [n.id for n in vi.all_nodes()]
    pick = nodes[:6] + nodes[len(nodes) // 2:len(nodes) // 2 + 4] + nodes[-6:]
    for i in pick:
        got = lv.fbm_brick(vi, i, seed, octaves=octaves, n_threads=3)
        want = oracle.fbm_brick(ovol, fp, i).view(np.uint8)
        assert np.array_equal(got, want), hex(i)


def test_fbm_threads_do_not_change_bytes(native):
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 32, 1, dtype=lv.DT_UINT16)
    node = [n.id for n in vi.all_nodes()][-1]
    one = lv.fbm_brick(vi, node, 5, n_threads=1)
    for t in (2, 7, 64):
        assert np.array_equal(lv.fbm_brick(vi, node, 5, n_threads=t), one)


def test_fbm_field_properties(oracle):
    # the permutation is a bijection: noise vanishes on integer lattice points
    for p in [(0, 0, 0), (3, 7, 250), (255, 1, 9)]:
        assert oracle.perlin(42, *p) == 0.0
    vals = [oracle.perlin(42, 0.37 * i, 0.11 * i, 0.73 * i) for i in range(1, 2000)]
    assert -1.0 <= min(vals) < -0.3 and 0.3 < max(vals) <= 1.0
    assert oracle.perlin(42, 1.5, 2.5, 3.5) != oracle.perlin(43, 1.5, 2.5, 3.5)


def test_fbm_invalid_arguments(native):
    import livre_gb300 as lv
    vi = lv.VolumeInformation(64, 16, 1)
    with pytest.raises(lv.LivreError):
        lv.fbm_brick(vi, lv.NodeId(0, (0, 0, 0)).id | 0xF, 1)   # level beyond the octree
    with pytest.raises(lv.LivreError):
        lv.fbm_brick(vi, 0, 1, octaves=0)
    with pytest.raises(lv.LivreError):
        lv.fbm_brick(vi, 0, 1, frequency=0.0)
