"""CPU check of the PyTorch-autograd reference used by the adjoint tests:
its autograd gradient of the extraction observable agrees with central
finite differences of itself."""
import numpy as np

from nrpytutorial_gb300.adjoint import ExtractionSphere
from tests.maxwell_torch_ref import TorchMaxwell


def test_torch_reference_gradient_matches_central_differences():
    sph = ExtractionSphere(1.6, ntheta=6, nphi=8)
    ref = TorchMaxwell(10, (-3.0, 3.0), sph.points, sph.weights, n_steps=5)
    amp, lam = 0.9, 1.3
    J, g = ref.gradient(amp, lam)
    h = 1e-6
    fd = np.array([(float(ref.observable(amp + h, lam)) - float(ref.observable(amp - h, lam))) / (2 * h),
                   (float(ref.observable(amp, lam + h)) - float(ref.observable(amp, lam - h))) / (2 * h)])
    assert J > 0
    assert np.allclose(g, fd, rtol=1e-6, atol=0), (g, fd)
