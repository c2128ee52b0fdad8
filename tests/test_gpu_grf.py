"""The device smoothing kernel (pmg_grf_smooth) reproduces the tensor
formulation of the GRF generator bit for bit, on batches of anisotropic
volumes and several smoothing orders, and batched media equal the
one-at-a-time generator."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [8, 24, 64])
def test_smoothing_kernel_equals_tensor_formulation(order):
    import torch

    from pmmoto_gb300.domain_generation import grf

    f = torch.stack([grf.noise((20, 33, 17), s) for s in (1, 2, 3)])
    assert torch.equal(grf.smooth_device(f, order), grf.smooth(f, order=order))


def test_batched_media_equal_single_media():
    import torch

    from pmmoto_gb300.domain_generation import grf
    from pmmoto_gb300.learned import data

    seeds, por = [11, 12, 13], np.array([0.3, 0.45, 0.6])
    batch = data.grf_batch(40, seeds, 3.0, por)
    for i, s in enumerate(seeds):
        one = grf.gen_grf_medium((40, 40, 40), porosity=float(por[i]), seed=s, sigma=3.0)
        assert torch.equal(batch[i], one)
        assert abs(one.float().mean().item() - por[i]) < 1e-4
