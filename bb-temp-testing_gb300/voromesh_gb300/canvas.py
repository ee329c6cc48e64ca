"""Python mirror of voromesh::Canvas (include/voromesh/canvas.h:25-89) over the
cv_* C ABI: the canvas lives on the GPU; the accessors copy to numpy.

RasterizeShape / StampDisc / TargetSlots / InsideMasks / IsInside / IsSurface
keep the reference's names and meaning (src/voromesh/canvas.cpp). One stated
difference: a stamp's new rim voxels take free slots in tile-major voxel
order, where the reference uses std::unordered_map order, so slot indices can
differ from the reference's by a relabelling.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, cv_edit, cv_info_t, load, ptr

TILE_LOG2 = 3
TILE_SIZE = 1 << TILE_LOG2


@dataclass
class Edit:
    """Canvas::Edit (canvas.h:38-45)."""
    dirtySlots: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    tx0: int = 0
    ty0: int = 0
    tx1: int = 0
    ty1: int = 0
    removed: int = 0
    added: int = 0
    flipped: int = 0

    def Changed(self) -> bool:
        return self.removed + self.added + self.flipped > 0


class Canvas:
    """voromesh::Canvas on one GPU."""

    kTileLog2 = TILE_LOG2
    kTileSize = TILE_SIZE

    def __init__(self, width: float, height: float, voxelSize: float):
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.cv_create(width, height, voxelSize, C.byref(h)), "Canvas")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.cv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> cv_info_t:
        i = cv_info_t()
        check(self._lib.cv_info(self._h, C.byref(i)), "Canvas.info")
        return i

    def RasterizeShape(self, polygon) -> float:
        """Returns the device milliseconds of the call."""
        a = np.ascontiguousarray(polygon, dtype=np.float32).reshape(-1, 2)
        ms = C.c_float()
        check(self._lib.cv_rasterize(self._h, ptr(a), len(a), C.byref(ms)), "RasterizeShape")
        return ms.value

    def StampDisc(self, center, radius: float, inside: bool, with_dirty: bool = True) -> Edit:
        e = cv_edit()
        check(self._lib.cv_stamp_disc(self._h, float(center[0]), float(center[1]), float(radius), int(bool(inside)),
                                      C.byref(e)), "StampDisc")
        out = Edit(tx0=e.tx0, ty0=e.ty0, tx1=e.tx1, ty1=e.ty1, removed=e.removed, added=e.added, flipped=e.flipped)
        if with_dirty and e.ndirty:
            d = np.zeros(e.ndirty, np.int32)
            check(self._lib.cv_edit_dirty(self._h, ptr(d), None, e.ndirty), "Edit.dirtySlots")
            out.dirtySlots = d
        return out

    def InDomain(self, i: int, j: int) -> bool:
        inf = self.info()
        return 0 <= i < inf.voxelsX and 0 <= j < inf.voxelsY

    def IsInside(self, i: int, j: int) -> bool:
        r = C.c_int()
        check(self._lib.cv_is_inside(self._h, i, j, C.byref(r)), "IsInside")
        return bool(r.value)

    def IsSurface(self, i: int, j: int) -> bool:
        r = C.c_int()
        check(self._lib.cv_is_surface(self._h, i, j, C.byref(r)), "IsSurface")
        return bool(r.value)

    def TargetSlots(self) -> np.ndarray:
        n = self.info().numSlots
        a = np.zeros((n, 2), np.float32)
        if n:
            check(self._lib.cv_get_slots(self._h, ptr(a)), "TargetSlots")
        return a

    def InsideMasks(self) -> np.ndarray:
        inf = self.info()
        m = np.zeros(inf.tilesX * inf.tilesY, np.uint64)
        check(self._lib.cv_get_inside(self._h, ptr(m)), "InsideMasks")
        return m

    def FreeSlots(self) -> np.ndarray:
        n = self.info().freeSlots
        f = np.zeros(max(n, 1), np.int32)
        check(self._lib.cv_get_free(self._h, ptr(f)), "FreeSlots")
        return f[:n]

    def Surface(self):
        """Dense surface: per-tile masks, per-voxel points and slots (tile-major)."""
        inf = self.info()
        tiles = inf.tilesX * inf.tilesY
        m = np.zeros(tiles, np.uint64)
        p = np.zeros((tiles * 64, 2), np.float32)
        s = np.zeros(tiles * 64, np.int32)
        check(self._lib.cv_get_surface(self._h, ptr(m), ptr(p), ptr(s)), "Surface")
        return m, p, s

    def state(self) -> dict:
        """The full state in one layout (as the oracle's Canvas.state())."""
        inf = self.info()
        m, p, s = self.Surface()
        return dict(slots=self.TargetSlots(), free=self.FreeSlots(), inside=self.InsideMasks(), smask=m, spt=p,
                    sslot=s, counts=(inf.numSlots, inf.freeSlots, int(inf.surfaceCount), inf.surfaceTiles))

    def TilesX(self) -> int: return self.info().tilesX
    def TilesY(self) -> int: return self.info().tilesY
    def VoxelSize(self) -> float: return self.info().voxelSize
    def SurfaceCount(self) -> int: return int(self.info().surfaceCount)
    def SurfaceTileCount(self) -> int: return self.info().surfaceTiles
