"""The tensor-core complex products (tcgen05, kind::tf32, split 3xTF32) that the FP32 stages of
the mixed form use: the same solve with them switched off (the SIMT FP32 kernel) agrees to
FP32-product rounding, both stay within the mixed form's 1e-6 of the reference's own run at the
crossed-grating sweep's full size (450 x 450 mode matrices), and no CTA's bounded wait on its
MMAs ran out."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), 'golden', 'ref_configs.npz')


def _solve(E, precision):
    d = np.load(FIX)
    names = [str(n) for n in d['names'] if str(n).startswith('crossed_')]
    cases = []
    for n in names:
        c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(n + '__')}
        cases.append(c)
    st = np.ascontiguousarray(d['crossed__structure'])
    conv = E.assemble(torch.as_tensor(st, device='cuda'), 7, 7)
    B, L = len(cases), st.shape[0]
    inp = E.BatchInputs([list(range(L))] * B, [list(np.asarray(c['thickness'], float)) for c in cases],
                        [float(c['wavelength']) for c in cases], [[1000.0, 1000.0]] * B, [0.0] * B, [0.0] * B,
                        [1.0] * B, [2.25] * B, [[1.0 + 0j, 0j]] * B)
    R, T, st_ = E.solve_batch(conv, inp, precision=precision)
    torch.cuda.synchronize()
    return cases, R.cpu().numpy(), T.cpu().numpy(), st_.cpu().numpy()


def test_mixed_form_with_and_without_tensor_cores():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import _lib, engine as E
    lib = _lib.load()
    try:
        lib.wb_set_tuning(_lib.WB_TUNE_TENSOR_CORES, 0)
        cases, R1, T1, s1 = _solve(E, 'mixed')
        lib.wb_set_tuning(_lib.WB_TUNE_TENSOR_CORES, 1)
        _, R0, T0, s0 = _solve(E, 'mixed')
    finally:
        lib.wb_set_tuning(_lib.WB_TUNE_TENSOR_CORES, 0)
    assert not (s1 & ~8).any() and not (s0 & ~8).any()
    assert int(lib.wb_tensor_core_errors()) == 0
    assert max(np.abs(R1 - R0).max(), np.abs(T1 - T0).max()) < 1e-7
    for b, c in enumerate(cases):
        for col, pol in ((1, 's'), (2, 'p')):
            scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
            for R in (R0, R1):
                assert np.abs(R[b, col] - c[f'R_{pol}']).max() < 1e-6 * scale
