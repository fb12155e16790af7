"""GB300-native narrow-band level-set advection (OpenVDB LevelSetAdvection /
LevelSetTracker hot path) behind a C ABI; see include/gbls.h."""
from . import _abi
from .fields import Field
from .grid import HostArena, HostGrid, bitwise_equal, compare, digest, summary, topology_equal
from .levelset import (FAST, FP64, PARITY, DeviceBatch, DeviceField, DeviceLevelSet, DeviceVolume, LevelSetAdvection,
                       LevelSetFilter, LevelSetMorphing, LevelSetTracker, VolumeAdvection)
