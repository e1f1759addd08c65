"""GB300 (sm_103a) FP64 residual / time-step path for the meshcfd finite-volume solver."""

__version__ = "0.1.0"
