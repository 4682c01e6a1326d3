"""Stand-in for the subset of the ``vtk`` package that JAXTrace's VTK reader
calls -- TEST INFRASTRUCTURE ONLY (lets the reference reader's own logic run
in a container without VTK when golden fixtures are regenerated).

The readers do not parse files: ``REGISTRY`` maps each absolute file path to
the dataset the fixture script wrote there (points and point-data arrays),
and ``GetOutput`` serves it through the accessors the reference calls
(io/vtk_reader.py:605-681).  What the reference then does with the data --
which files it picks and in which order, which array it takes as the
velocity, how it pads components, the bounds and the time values -- is its
own code, and that is what the fixtures record.
"""
from __future__ import annotations

import os

import numpy as _np

# absolute path -> {"points": (N, 3), "point_data": [(name, array), ...]}
REGISTRY: dict = {}


class _Array:
    def __init__(self, a):
        self.a = _np.asarray(a)

    def GetNumberOfComponents(self):
        return 1 if self.a.ndim == 1 else int(self.a.shape[1])

    def GetNumberOfTuples(self):
        return int(self.a.shape[0])


class _FieldData:
    def __init__(self, arrays):
        self.arrays = list(arrays)

    def GetNumberOfArrays(self):
        return len(self.arrays)

    def GetArrayName(self, i):
        return self.arrays[i][0]

    def GetArray(self, key):
        if isinstance(key, int):
            return _Array(self.arrays[key][1]) if 0 <= key < len(self.arrays) else None
        for name, a in self.arrays:
            if name == key:
                return _Array(a)
        return None


class _Points:
    def __init__(self, p):
        self.p = p

    def GetData(self):
        return _Array(self.p)


class _Output:
    def __init__(self, entry):
        self.e = entry

    def GetPoints(self):
        return _Points(self.e["points"])

    def GetPointData(self):
        return _FieldData(self.e["point_data"])

    def GetCellData(self):
        return _FieldData([])

    def GetNumberOfPoints(self):
        return int(len(self.e["points"]))

    def GetBounds(self):
        p = _np.asarray(self.e["points"], dtype=_np.float64)
        lo, hi = p.min(axis=0), p.max(axis=0)
        return (lo[0], hi[0], lo[1], hi[1], lo[2], hi[2])


class _Reader:
    def __init__(self):
        self.name = None

    def SetFileName(self, name):
        self.name = name

    def Update(self):
        if os.path.abspath(self.name) not in REGISTRY:
            raise OSError(f"no registered dataset for {self.name}")

    def GetOutput(self):
        return _Output(REGISTRY[os.path.abspath(self.name)])


class vtkXMLUnstructuredGridReader(_Reader):
    pass


class vtkXMLPUnstructuredGridReader(_Reader):
    pass


class vtkUnstructuredGridReader(_Reader):
    pass
