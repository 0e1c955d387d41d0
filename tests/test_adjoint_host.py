"""Host-side argument checks of the differentiable step and the analytic
fields (no GPU needed)."""
import pytest


def test_advect_rejects_unknown_checkpoint_mode():
    pytest.importorskip("torch")
    from tbslas_gb300 import adjoint
    with pytest.raises(ValueError, match="checkpoint"):
        adjoint.advect(None, None, None, None, 0.01, 1, 1, 0, checkpoint="midpoints")


def test_field_parameter_counts_checked_on_the_host():
    """The C ABI reads the kind's parameter count from the array; the Python
    face refuses arrays of another length before any call."""
    import numpy as np
    import tbslas_gb300 as tb
    assert tb.Field.gaussians([(0.5, 0.5, 0.5), (0.2, 0.3, 0.4)], 0.1).params.size == 10
    assert tb.Field.taylor_green().params.size == 0
    assert tb.Field(tb.Field.HOPF, [0.5, 0.5, 0.5, 1.0, 0.1]).dof == 3
    with pytest.raises(ValueError, match="parameters"):
        tb.Field(tb.Field.GAUSSIAN_3D, [0.5, 0.5])
    with pytest.raises(ValueError, match="parameters"):
        tb.Field(tb.Field.FOURIER, np.zeros(9), n=2)
    assert tb.Field(11).params.size == 0  # unknown kinds are the C ABI's to reject
