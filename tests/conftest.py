import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (runs through the C-ABI library)')


#: Modules collected after every other one, in their own (alphabetical) order: incidence from
#: below and by wavevector, the ETM and field paths, gain films, which sit on top of the parity-tested stages, the amplitude ratios, the half-space
#: branches, the RETICOLO orders, the wavelength gradient and the serving loop's integrated
#: coefficients, so that under ``-x`` a failure there cannot keep the stage-level parity suites
#: from reporting; and the allocation-free entry point, whose fixed scratch is shared by the
#: whole process, at the end.
_LAST = ('test_backside.py', 'test_direct_incidence.py', 'test_etm.py', 'test_fields.py', 'test_gain_film.py', 'test_gpu_amplitudes.py', 'test_gpu_halfspace.py',
         'test_gpu_reticolo.py', 'test_gpu_wavelength_gradient.py', 'test_serving_integrated.py',
         'test_zz_no_alloc.py')


def pytest_collection_modifyitems(session, config, items):
    items.sort(key=lambda item: os.path.basename(str(item.fspath)) in _LAST)
