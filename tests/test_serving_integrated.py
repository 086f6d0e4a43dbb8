"""The serving loop with integrated (closed-form segment) Li coefficients: each layer's raster
is compressed on the host and assembled by wb_assemble_li_integrated; results against the
oracle's solve on integrated slots."""
import numpy as np
import pytest

from wavebit_gb300.serving import Server


@pytest.mark.gpu
def test_integrated_coefficients_are_served_like_the_oracle():
    """A backend built with integrated coefficients assembles compressed cells; its results
    equal the oracle's solve on integrated slots."""
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from oracle import rcwa_oracle as O
    from wavebit_gb300.serving import GpuBackend, _stream
    reqs = _stream(6, rate=400.0, seed=21, orders=[(2, 2), (3, 3)], max_layers=2, sides=(32,))
    got, st = Server(GpuBackend(2, 6 << 30, coefficients='integrated'), n_workers=2, max_batch=4).run(reqs)
    assert st['completed'] == len(reqs)
    for r in reqs:
        hu, hv = r.orders
        o = O.solve_stack(r.eps, r.thickness, r.wavelength, r.period, hu, hv, r.theta, r.phi, r.eps_top,
                          r.eps_bot, r.pol, conv=O.to_conv_mat_raster_integrated(r.eps, hu, hv))
        a = got[r.id]
        scale = max(np.abs(o['R'][0]).max(), np.abs(o['T'][0]).max())
        assert np.abs(a.R - o['R'][0]).max() <= 1e-10 * scale and np.abs(a.T - o['T'][0]).max() <= 1e-10 * scale
