"""The oracle's Kelvinlet restatement against the reference's compiled
kelvinlet.c (CPU): grab, grab_biscale, grab_triscale, scale and twist with
BKE_kelvinlet_init_params, bit for bit on seeded inputs."""
import numpy as np
import pytest

import pyrefpin

pytestmark = pytest.mark.skipif(not pyrefpin.available(),
                                reason="reference tree absent: the pinning library cannot be built")


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
def test_kelvinlet_matches_reference(oracle, kind):
    rng = np.random.default_rng(0x5EED0000 + 70 + kind)
    for _ in range(400):
        radius = np.float32(rng.uniform(0.02, 0.5))
        force = np.float32(rng.normal() * 0.3)
        poisson = np.float32(rng.uniform(0.0, 0.9))
        co = rng.normal(size=3).astype(np.float32) * 0.3
        loc = rng.normal(size=3).astype(np.float32) * 0.3
        dn = rng.normal(size=3).astype(np.float32)
        if kind >= 3:
            dn = (dn / np.linalg.norm(dn)).astype(np.float32)
        a = oracle.kelvinlet(kind, radius, force, poisson, co, loc, dn)
        b = pyrefpin.kelvinlet(kind, radius, force, poisson, co, loc, dn)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (kind, a, b)
    # the element at the brush centre
    z = np.zeros(3, np.float32)
    a = oracle.kelvinlet(kind, 0.1, 0.5, 0.4, z, z, np.array([0, 0, 1], np.float32))
    b = pyrefpin.kelvinlet(kind, 0.1, 0.5, 0.4, z, z, np.array([0, 0, 1], np.float32))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
