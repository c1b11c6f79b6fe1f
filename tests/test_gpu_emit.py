"""Device emission (MPM.add of a box, sphere or cylinder sampled on the GPU) against the host
sampler and record conversion (sampleShape + add(), mpm.js:207-232, 683-714): the same records,
bit for bit, including truncation at maxParticles and large lattices."""
import numpy as np
import pytest

from shaderintel_gb300 import MPM

pytestmark = pytest.mark.gpu

CASES = [
    ({"box": [[0.1, 0.12, 0.13], [0.61, 0.55, 0.47]]}, dict(material="water", velocity=[0.3, -1, 0.2])),
    ({"sphere": [[0.5, 0.45, 0.52], 0.23]}, dict(material="jelly", seed=12345, jitter=0.9)),
    ({"cylinder": [[0.4, 0.5, 0.6], 0.17, 0.2]}, dict(material="snow", velocity=[0, 0, -2], seed=7)),
    ({"box": [[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]]}, dict(material="sand", jitter=0.0)),    # clamped to the walls
]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("k", range(len(CASES)))
def test_device_emission_equals_host_sampling(k):
    shape, opts = CASES[k]
    dev = MPM(grid=40, maxParticles=600000, substeps=6, origin=[0.05, -0.1, 0.2], size=[1.2, 1.0, 1.1])
    host = MPM(grid=40, maxParticles=600000, substeps=6, origin=[0.05, -0.1, 0.2], size=[1.2, 1.0, 1.1])
    dev.add({"box": [[0.2, 0.2, 0.2], [0.3, 0.3, 0.3]]}, material="honey")          # emission appends
    host.add({"box": [[0.2, 0.2, 0.2], [0.3, 0.3, 0.3]]}, material="honey", _host=True)
    n_dev = dev.add(shape, **opts)
    n_host = host.add(shape, _host=True, **opts)
    assert n_dev == n_host > 0
    assert np.array_equal(bits(dev.readParticles()), bits(host.readParticles()))
    dev.destroy()
    host.destroy()


def test_device_emission_truncates_at_capacity_and_steps():
    dev = MPM(grid=64, maxParticles=100000, substeps=8)
    host = MPM(grid=64, maxParticles=100000, substeps=8)
    shape = {"box": [[0.05, 0.05, 0.05], [0.95, 0.5, 0.95]]}     # ~1.4 M lattice points, keeps 100k
    assert dev.add(shape, material="water") == host.add(shape, material="water", _host=True) == 100000
    assert dev.add({"sphere": [[0.5, 0.8, 0.5], 0.1]}) == 0
    assert np.array_equal(bits(dev.readParticles()), bits(host.readParticles()))
    dev.step()
    host.step()
    assert np.array_equal(bits(dev.readParticles()), bits(host.readParticles()))
    dev.destroy()
    host.destroy()
