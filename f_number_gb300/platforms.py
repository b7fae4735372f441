"""Platform switch (``+platforms/**``): ``gpu(index)`` runs the CUDA library.

``cpu`` names the reference's MATLAB loop (``das_pw.m:302-481``); this package
implements the ``platforms.gpu`` path only, so ``das_pw(..., platforms.cpu())``
raises instead of falling back to a CPU implementation.
"""
from __future__ import annotations


class platform:
    def __str__(self):
        return self.string()


class cpu(platform):
    def string(self):
        return "cpu"


class gpu(platform):
    def __init__(self, index: int = 0):
        index = int(index)
        if index < 0:
            raise ValueError("index must be nonnegative")
        self.index = index

    def string(self):
        return "gpu_%d" % self.index
