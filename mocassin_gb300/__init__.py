"""GB300-native Monte Carlo energy-packet transport for mocassin.

Drop-in for mocassin's packet loop (``energyPacketDriver``, the ray march
``pathSegment`` and the Jste/Jdif path-length estimators) behind the C-ABI of
``include/mocassin_gpu.h``; see ``transport.energy_packet_driver``.
"""
from . import abi, nebula  # noqa: F401

__all__ = ["abi", "nebula", "transport", "build"]
