"""Learned radius schedule for the drainage sweep (no counterpart in the
reference): a small 3-D CNN over the downsampled distance field predicts the
saturation curve, and the exact drainage evaluates only the radii where that
curve moves (``schedule``); the network runs on the project's own bf16
tensor-core convolution kernels for inference and training (``net``)."""

from .net import ScheduleNet  # noqa: F401

__all__ = ["ScheduleNet"]
