"""Host-side argument checks of the differentiable step (no GPU needed)."""
import pytest


def test_advect_rejects_unknown_checkpoint_mode():
    pytest.importorskip("torch")
    from tbslas_gb300 import adjoint
    with pytest.raises(ValueError, match="checkpoint"):
        adjoint.advect(None, None, None, None, 0.01, 1, 1, 0, checkpoint="midpoints")
