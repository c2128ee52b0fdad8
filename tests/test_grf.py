"""The Gaussian-random-field generator is reproducible bit for bit: the
package's torch implementation (run here on the CPU, the same operations the
device runs) equals the independent C host twin that made the 1024^3 fixture
(tests/golden/grf_host.c), field and medium, on several shapes and seeds."""

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))


@pytest.mark.parametrize("shape,seed", [((32, 40, 36), 7), ((20, 70, 33), 3), ((65, 16, 24), 11)])
def test_torch_generator_equals_host_twin(shape, seed):
    import grf as host

    from pmmoto_gb300.domain_generation import grf

    f_host = host.grf_field_host(shape, seed)
    f_dev = grf.grf_field(shape, seed, device="cpu").numpy()
    assert np.array_equal(f_host, f_dev)
    m_host = host.grf_medium_host(shape, 0.35, seed)
    m_dev = grf.gen_grf_medium(shape, 0.35, seed, device="cpu").numpy()
    assert np.array_equal(m_host, m_dev)
    assert abs(m_host.mean() - 0.35) < 1e-3


def test_binomial_kernel_has_the_gaussian_variance():
    from pmmoto_gb300.domain_generation import grf

    w = np.array(grf.binomial_weights())
    k = np.arange(len(w)) - grf.HALF
    assert abs(w.sum() - 1.0) < 1e-15
    assert abs((w * k * k).sum() - 16.0) < 1e-12  # sigma = 4 voxels
