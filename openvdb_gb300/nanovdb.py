"""NanoVDB buffers of level sets (nanovdb::tools::createNanoGrid for FloatGrids).

to_nanovdb(grid) returns the NanoGrid<float> buffer (NanoVDB 32.9,
breadth-first) of a HostGrid as a uint8 numpy array: byte for byte what
createNanoGrid(openvdb::FloatGrid, StatsMode, CheckMode) writes
(nanovdb/tools/CreateNanoGrid.h:162-168), so NanoVDB readers, renderers and
GPU samplers take it unchanged.  to_device(grid) places the same buffer in
device memory (a torch uint8 tensor) for CUDA consumers of NanoVDB.

export_device(level_set) and export_index_device(level_set) write the
buffers on the device straight from a DeviceLevelSet (or a DeviceBatch
instance), the same bytes as the host exporters of its downloaded grid;
from_device(buffer) makes a DeviceLevelSet from a NanoGrid<float> buffer in
device (or host) memory, its leaves gathered on the device.
"""
import ctypes as C

import numpy as np

from ._lib import check, lib

STATS = {"disable": 0, "bbox": 1, "minmax": 2, "all": 3}
CHECKSUM = {"disable": 0, "partial": 1, "full": 2}


def to_nanovdb(grid, name="", stats="all", checksum="partial"):
    """NanoGrid<float> buffer of `grid` (a HostGrid) named `name`."""
    L = lib()
    d = grid.desc()
    n = C.c_int64()
    s, c = STATS[stats], CHECKSUM[checksum]
    nm = name.encode()
    check(L.gbls_nanovdb_export(C.byref(d), nm, s, c, None, 0, C.byref(n)), host=True)
    buf = np.empty(n.value, np.uint8)
    check(L.gbls_nanovdb_export(C.byref(d), nm, s, c, buf.ctypes.data, n.value, C.byref(n)), host=True)
    return buf


def to_nanovdb_index(grid, name="", channel=True, include_stats=True, include_tiles=True,
                     checksum="partial"):
    """NanoGrid<ValueOnIndex> buffer of `grid` (createNanoGrid<FloatGrid,
    ValueOnIndex>(grid, channels, includeStats, includeTiles)); with
    `channel` the values follow as the blind-data array "channel_0"."""
    L = lib()
    d = grid.desc()
    n = C.c_int64()
    args = (name.encode(), int(bool(channel)), int(bool(include_stats)), int(bool(include_tiles)),
            CHECKSUM[checksum])
    check(L.gbls_nanovdb_export_index(C.byref(d), *args, None, 0, C.byref(n)), host=True)
    buf = np.empty(n.value, np.uint8)
    check(L.gbls_nanovdb_export_index(C.byref(d), *args, buf.ctypes.data, n.value, C.byref(n)), host=True)
    return buf


def from_nanovdb(buffer):
    """HostGrid of a NanoGrid<float> buffer (bytes or a uint8 array)."""
    from .fixtures import _from_native
    a = np.ascontiguousarray(np.frombuffer(bytes(buffer), np.uint8) if isinstance(buffer, (bytes, bytearray))
                             else buffer, dtype=np.uint8)
    h = C.c_void_p()
    check(lib().gbls_nanovdb_import(a.ctypes.data, a.size, C.byref(h)), host=True)
    return _from_native(h)


def to_device(grid, name="", stats="all", checksum="partial", device="cuda"):
    """The same buffer as a torch uint8 tensor on `device`."""
    import torch
    return torch.from_numpy(to_nanovdb(grid, name, stats, checksum)).to(device)


def _device_buffer(level_set, fn, args):
    """Size query, allocation and fill of a device buffer by a
    gbls_nanovdb_export*_device entry point."""
    import torch
    L = lib()
    n = C.c_int64()
    check(fn(level_set.handle, *args, None, 0, C.byref(n)))
    dev = torch.device("cuda", getattr(level_set, "device", 0))
    buf = torch.empty(n.value, dtype=torch.uint8, device=dev)
    torch.cuda.current_stream(dev).synchronize()  # the allocation may reuse memory of pending work
    check(fn(level_set.handle, *args, C.c_void_p(buf.data_ptr()), n.value, C.byref(n)))
    return buf


def export_device(level_set, name="", stats="all", checksum="partial", instance=-1):
    """NanoGrid<float> of a DeviceLevelSet (instance -1) or of instance i of a
    DeviceBatch, written on the device: a torch uint8 CUDA tensor."""
    L = lib()
    return _device_buffer(level_set, L.gbls_nanovdb_export_device,
                          (int(instance), name.encode(), STATS[stats], CHECKSUM[checksum]))


def export_index_device(level_set, name="", channel=True, include_stats=True, include_tiles=True,
                        checksum="partial", instance=-1):
    """NanoGrid<ValueOnIndex> (with the value channel) of a device level set,
    written on the device."""
    L = lib()
    return _device_buffer(level_set, L.gbls_nanovdb_export_index_device,
                          (int(instance), name.encode(), int(bool(channel)), int(bool(include_stats)),
                           int(bool(include_tiles)), CHECKSUM[checksum]))


def from_device(buffer, device=0):
    """DeviceLevelSet of a NanoGrid<float> buffer: a torch uint8 tensor (CUDA
    or CPU) or a numpy array."""
    import struct
    from .levelset import DeviceLevelSet, _call
    L = lib()
    try:
        import torch
        is_tensor = isinstance(buffer, torch.Tensor)
    except ImportError:
        is_tensor = False
    if is_tensor:
        if buffer.dtype != torch.uint8 or not buffer.is_contiguous():
            raise ValueError("a contiguous uint8 tensor is expected")
        if buffer.is_cuda:
            torch.cuda.current_stream(buffer.device).synchronize()
        ptr, size = buffer.data_ptr(), buffer.numel()
        head = bytes(buffer[:min(size, 800)].cpu().numpy())
        keep = buffer
    else:
        a = np.ascontiguousarray(buffer, dtype=np.uint8)
        ptr, size = a.ctypes.data, a.size
        head = a[:800].tobytes()
        keep = a
    _call(L.gbls_set_device(int(device)))
    h = C.c_void_p()
    _call(L.gbls_create_from_nanovdb(C.c_void_p(ptr), size, C.byref(h)))
    del keep
    # the map's scale (the double matrix) and the root's background
    voxel_size = struct.unpack_from("<d", head, 296 + 88)[0]
    root_at = 672 + struct.unpack_from("<q", head, 672 + 24)[0]
    background = struct.unpack_from("<f", head, root_at + 28)[0] if root_at + 32 <= len(head) else None
    return DeviceLevelSet._adopt(h, voxel_size, background, device)


def probe(buffer, ijk):
    """nanovdb::ReadAccessor getValue / isActive on a device NanoVDB buffer
    (torch uint8 CUDA tensor) at index coordinates ijk (int32 CUDA tensor,
    n x 3): (float32 values of a NanoGrid<float> or int64 value indices of a
    NanoGrid<ValueOnIndex>, uint8 active flags), CUDA tensors."""
    import torch
    L = lib()
    c = ijk.to(dtype=torch.int32).contiguous()
    n = c.shape[0]
    is_float = int(buffer[636:640].cpu().numpy().view(np.uint32)[0]) == 1
    out = torch.empty(n, dtype=torch.float32 if is_float else torch.int64, device=buffer.device)
    act = torch.empty(n, dtype=torch.uint8, device=buffer.device)
    stream = torch.cuda.current_stream(buffer.device)
    ptr = C.c_void_p(out.data_ptr())
    check(L.gbls_nanovdb_probe(C.c_void_p(buffer.data_ptr()), buffer.numel(), C.c_void_p(c.data_ptr()), n,
                               ptr if is_float else None, None if is_float else ptr, C.c_void_p(act.data_ptr()),
                               C.c_void_p(stream.cuda_stream)))
    return out, act

