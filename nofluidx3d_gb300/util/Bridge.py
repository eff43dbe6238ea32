"""Bridge: a host array mirrored by device state (nofluidx3d/util/Bridge.py:16-26).

In the reference a Bridge owns an OpenCL buffer. Here the device state lives in the nfx_sim
handle in its own (reordered, FP32 hi/lo) layout, so a Bridge is a host array plus the getter
and setter of the handle that convert to and from the reference layout (SoA float64).
"""

from __future__ import annotations

from typing import Callable

import numpy as np


class Bridge:
    def __init__(self, startarray, datatype, read: Callable | None = None, write: Callable | None = None):
        self.arrayC = np.asarray(startarray).astype(datatype)
        self._read = read
        self._write = write

    def readFromGPU(self):
        if self._read is not None:
            self._read(self.arrayC)
        return self.arrayC

    def writeToGPU(self):
        if self._write is None:
            raise NotImplementedError("this buffer is read-only on the device")
        self._write(self.arrayC)
