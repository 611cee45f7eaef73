"""GB300-native exciton path of WTB: H(k) and bands, BSE operator, lowest-exciton solve, spectrum.

``wtb_gb300.api`` binds the C ABI of ``libwtb_gb300.so`` (declared in ``include/wtb_gpu.h``);
``wtb_gb300.synthetic`` builds the seeded tight-binding inputs.
"""
from . import synthetic  # noqa: F401

__all__ = ["synthetic", "api"]
