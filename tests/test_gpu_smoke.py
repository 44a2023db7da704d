"""The package's smoke check (one small blob update on the GPU against the
oracle, FP64 and the mixed-precision learned path, one network forward and
backward pass) as a test, so that the suite runs it too."""
import pytest

pytestmark = pytest.mark.gpu


def test_smoke(gpulib):
    import __graft_entry__ as g
    g.smoke()
