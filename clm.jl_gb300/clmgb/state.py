"""Structure-of-arrays column state, host (numpy) or device (torch CUDA tensors).

Each field is stored exactly as CLM.jl stores it: a Julia column-major
``Matrix{Float64}(nc, nlev)`` becomes an array of shape ``(nlev, ldc)`` whose
row ``jj-1`` holds level ``jj`` for all columns, so the device pointer handed to
the C ABI addresses element ``(c, jj)`` at ``c + (jj-1)*ldc``.  Column vectors
are shape ``(nc,)``, patch matrices ``(nlev, ldp)``.
"""
import ctypes as C

import numpy as np

from . import abi

_NP = {"u8": np.uint8, "i64": np.int64, "f64": np.float64}


def field_shape(name_kind_dims, vp, nc, npch, nl):
    _, _, kind, dims = name_kind_dims
    n = {"c": nc, "p": npch, "l": nl}[kind]
    if dims is None:
        return (n,)
    return (abi.level_count(dims, vp), n)


class ColumnState:
    """All fields of the soil/snow column solve for `nc` columns."""

    def __init__(self, vp, nc, npch=None, nl=1, arrays=None):
        self.vp = vp
        self.nc = int(nc)
        self.np = int(nc if npch is None else npch)
        self.nl = int(nl)
        self.arrays = {}
        spec = {f[0]: f for f in abi.all_fields()}
        self.spec = spec
        if arrays is None:
            for name, f in spec.items():
                self.arrays[name] = np.zeros(field_shape(f, vp, self.nc, self.np, self.nl), dtype=_NP[f[1]])
        else:
            self.arrays = arrays

    # ---- container helpers ----
    def __getitem__(self, k):
        return self.arrays[k]

    def __setitem__(self, k, v):
        self.arrays[k] = v

    @property
    def on_device(self):
        a = next(iter(self.arrays.values()))
        return not isinstance(a, np.ndarray)

    def bounds(self):
        return abi.Bounds(self.nc, self.np, self.nl, self.nc, self.np)

    def copy(self):
        if self.on_device:
            arrs = {k: v.clone() for k, v in self.arrays.items()}
        else:
            arrs = {k: v.copy() for k, v in self.arrays.items()}
        return ColumnState(self.vp, self.nc, self.np, self.nl, arrs)

    def to_device(self, device="cuda"):
        import torch
        arrs = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in self.arrays.items()}
        return ColumnState(self.vp, self.nc, self.np, self.nl, arrs)

    def to_host(self):
        if not self.on_device:
            return self.copy()
        arrs = {k: v.detach().cpu().numpy().copy() for k, v in self.arrays.items()}
        return ColumnState(self.vp, self.nc, self.np, self.nl, arrs)

    def subset(self, cols):
        """Host copy restricted to column indices `cols` (one patch per column layouts only)."""
        assert not self.on_device and self.np == self.nc
        cols = np.asarray(cols)
        out = {}
        for name, f in self.spec.items():
            a = self.arrays[name]
            if f[2] in ("c", "p"):
                out[name] = np.ascontiguousarray(a[..., cols])
            else:
                out[name] = a.copy()
        st = ColumnState(self.vp, len(cols), len(cols), self.nl, out)
        idx = np.arange(1, len(cols) + 1, dtype=np.int64)
        st["col_patchi"][:] = idx
        st["col_patchf"][:] = idx
        st["patch_column"][:] = idx
        return st

    # ---- ABI structs ----
    def _ptr(self, name, ctype):
        a = self.arrays[name]
        if isinstance(a, np.ndarray):
            assert a.flags.c_contiguous, name
            return a.ctypes.data_as(ctype)
        assert a.is_contiguous(), name
        return C.cast(C.c_void_p(a.data_ptr()), ctype)

    def _struct(self, cls, fields):
        s = cls()
        s.struct_size = C.sizeof(cls)
        for (n, t, _, _) in fields:
            setattr(s, n, self._ptr(n, abi._CT[t]))
        return s

    def soiltemp_fields(self):
        return self._struct(abi.SoilTempFields, abi.SOILTEMP_FIELDS)

    def soilwater_fields(self):
        return self._struct(abi.SoilWaterFields, abi.SOILWATER_FIELDS)

    def ptr(self, name):
        f = self.spec[name]
        return self._ptr(name, abi._CT[f[1]])


class ColumnRange:
    """The columns [c0, c1) of a device state, as the drop-in calls see them: column
    pointers advanced by c0 (same ldc), patch and landunit arrays whole.  A caller that
    runs the calls on a range also sets CLMGB_OPT_COLUMN_BASE to c0, since patch.column
    holds global column indices."""
    on_device = True

    def __init__(self, dev, c0, c1):
        self.dev, self.c0, self.c1 = dev, c0, c1

    def bounds(self):
        b = self.dev.bounds()
        return abi.Bounds(self.c1 - self.c0, b.np, b.nl, b.ldc, b.ldp)

    def _struct(self, cls, fields):
        st = cls()
        st.struct_size = C.sizeof(cls)
        for (n, t, kind, _) in fields:
            a = self.dev[n]
            off = self.c0 * a.element_size() if kind == "c" else 0
            setattr(st, n, C.cast(C.c_void_p(a.data_ptr() + off), abi._CT[t]))
        return st

    def soiltemp_fields(self):
        return self._struct(abi.SoilTempFields, abi.SOILTEMP_FIELDS)

    def soilwater_fields(self):
        return self._struct(abi.SoilWaterFields, abi.SOILWATER_FIELDS)
