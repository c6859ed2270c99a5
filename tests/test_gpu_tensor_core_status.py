"""Failure detection of the tensor-core kernels without a GPU fault.

Every wait in the tcgen05 kernels is bounded; a wait that gives up sets a bit in the mesh's status
word, the CTA drains and frees its tensor memory, and the host reports the failure at the next
synchronisation.  The self-test entry point makes one wait run out (an mbarrier phase that nothing
completes, short bound) and the test checks the reported error and that the mesh keeps working.
"""
import numpy as np
import pytest

from jgcm import configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp32", "tf32x3"])
def test_bounded_wait_reports_and_recovers(jg, orc, prec):
    gm = jg.Spectral_Spherical_Mesh(21, 22, 32, 64, 2, 6371.0e3, precision=prec)
    st = jg.lib().jgcm_selftest_bounded_wait(gm._h)
    assert st == -2  # JGCM_E_CUDA
    assert b"gave up waiting" in jg.lib().jgcm_last_error()
    # the status bit is cleared and the mesh still transforms correctly
    om = orc.Spectral_Spherical_Mesh(21, 22, 32, 64, 2, 6371.0e3)
    rng = np.random.default_rng(1)
    g = np.asfortranarray(rng.standard_normal((64, 32, 2)))
    a, b = gm.spectral(2), om.spectral(2)
    jg.Trans_Grid_To_Spherical(gm, g, a)
    orc.Trans_Grid_To_Spherical(om, g, b)
    assert configs.rel_l2(a, b) < 2e-5
