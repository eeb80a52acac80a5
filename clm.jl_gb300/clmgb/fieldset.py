"""A set of CLM fields described by an (name, type, kind, levels) spec, host (numpy)
or device (torch), with the matching ABI struct of pointers.  Column level arrays
are (levels, ldc) as CLM.jl's column-major [nc, levels] matrices; patch ones
(levels, ldp).  Kinds: 'c' column, 'p' patch, 'l' landunit, 'g' gridcell."""
import ctypes as C

import numpy as np

from . import abi

_NP = {"u8": np.uint8, "i64": np.int64, "f64": np.float64}


class FieldSet:
    SPEC = ()
    STRUCT = None

    def __init__(self, vp, nc, npch=None, nl=1, arrays=None, ng=1):
        self.vp, self.nc = vp, int(nc)
        self.np = int(nc if npch is None else npch)
        self.nl, self.ng = int(nl), int(ng)
        if arrays is None:
            arrays = {}
            for (n, t, kind, dims) in self.SPEC:
                m = {"c": self.nc, "p": self.np, "l": self.nl, "g": self.ng}[kind]
                shape = (m,) if dims is None else (abi.level_count(dims, vp), m)
                arrays[n] = np.zeros(shape, dtype=_NP[t])
        self.arrays = arrays

    def __getitem__(self, k):
        return self.arrays[k]

    def __setitem__(self, k, v):
        self.arrays[k] = v

    def _like(self, arrays):
        return type(self)(self.vp, self.nc, self.np, self.nl, arrays, ng=self.ng)

    def bounds(self):
        return abi.Bounds(self.nc, self.np, self.nl, self.nc, self.np)

    def to_device(self, device="cuda"):
        import torch
        return self._like({k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in self.arrays.items()})

    def to_host(self):
        return self._like({k: (v if isinstance(v, np.ndarray) else v.detach().cpu().numpy()).copy()
                           for k, v in self.arrays.items()})

    def copy(self):
        return self._like({k: (v.copy() if isinstance(v, np.ndarray) else v.clone()) for k, v in self.arrays.items()})

    def fields(self, skip=()):
        s = self.STRUCT()
        s.struct_size = C.sizeof(self.STRUCT)
        for (n, t, _, _) in self.SPEC:
            if n in skip:
                continue
            a = self.arrays[n]
            if isinstance(a, np.ndarray):
                assert a.flags.c_contiguous, n
                p = a.ctypes.data_as(abi._CT[t])
            else:
                assert a.is_contiguous(), n
                p = C.cast(C.c_void_p(a.data_ptr()), abi._CT[t])
            setattr(s, n, p)
        return s
