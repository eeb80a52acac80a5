"""Column steps for a caller whose state lives in host memory.

A driver that keeps CLM's arrays on the host (the reference's CPU runs) calls the
drop-in entry points on a device mirror of its state.  HostStepper keeps that mirror
and moves, per step, only what has to move:

* STATIC fields (geometry, soil parameters, column/patch topology) are uploaded once;
  the rest of the model does not change them between steps.
* INPUTS, the fields the step reads that the rest of the model changes between steps
  (prognostic state, forcing, snow bookkeeping), go host -> device before each step.
  Fields the step writes before it reads them (fact, thk, imelt, smp_l, ...) do not.
* Every field the step writes comes back device -> host.  Those that are final once
  soil_temperature! and set_soil_water_fractions! have run are read back on a second
  stream while the Richards solve runs; the Richards outputs follow it.

With chunks > 1 (step_chunked) soil_temperature! and set_soil_water_fractions! run
over column ranges: the inputs of range i+1 go up while range i computes, and the
temperature outputs of range i come back while the next ranges and the Richards
solve run; the Richards solve itself covers all columns in one call.  Column fields
move as strided rows of their [ldc, levels] layout (clmgb_copy_columns); the calls
see a range through column pointers advanced by its first column and
CLMGB_OPT_COLUMN_BASE.  Columns are independent, so the results do not depend on
the chunking.

The arithmetic is the device step's: the host arrays end up bit for bit as a
device-resident run leaves its state (tests/test_gpu_hoststep.py).
"""
import ctypes as C

import numpy as np

from . import abi, api

STATIC = ("mask_nolakec", "mask_nolakep", "mask_hydrology", "col_nbedrock", "col_itype", "col_landunit",
          "col_patchi", "col_patchf", "lun_itype", "lun_urbpoi", "patch_column", "patch_landunit", "patch_wtcol",
          "dz", "z", "zi", "watsat", "bsw", "sucsat", "hksat", "tkmg", "tkdry", "csol", "smpmin")

INPUTS = ("col_snl", "frac_veg_nosno", "t_soisno", "t_h2osfc", "t_grnd", "emg", "htvp", "eflx_bot", "dlrad", "cgrnd",
          "eflx_sh_grnd", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc", "h2osoi_liq", "h2osoi_ice", "excess_ice",
          "h2osno_no_layers", "h2osfc", "int_snow", "frac_sno_eff", "frac_h2osfc", "snow_depth", "snomelt_accum",
          "qflx_evap_soi", "qflx_ev_snow", "qflx_ev_soil", "qflx_ev_h2osfc", "sabg", "sabg_soil", "sabg_snow",
          "sabg_lyr", "forc_lwrad", "qflx_rootsoi", "qflx_infl", "zwt", "num_substeps")

# written by soil_temperature! / set_soil_water_fractions! (and the forcing injection);
# final before the Richards solve starts
WRITTEN_TEMPERATURE = ("t_soisno", "h2osoi_ice", "t_h2osfc", "t_grnd", "fact", "thk", "imelt", "xmf", "xmf_h2osfc",
                       "c_h2osfc", "eflx_fgr12", "eflx_fgr", "eflx_snomelt", "eflx_snomelt_r", "eflx_snomelt_u",
                       "eflx_h2osfc_to_snow", "eflx_gnet", "dgnetdT", "sabg_chk", "excess_ice", "h2osno_no_layers",
                       "h2osfc", "int_snow", "snow_depth", "bw", "exice_subs", "snomelt_accum", "qflx_snomelt",
                       "qflx_snofrz", "qflx_snow_drain", "qflx_h2osfc_to_ice", "qflx_snomelt_lyr", "qflx_snofrz_lyr",
                       "eff_porosity", "icefrac", "forc_lwrad", "qflx_infl", "sabg", "sabg_soil", "sabg_snow",
                       "sabg_lyr")
# written by the Richards solve
WRITTEN_WATER = ("h2osoi_liq", "qcharge", "smp_l", "hk_l", "num_substeps")


_KIND = {n: k for (n, _, k, _) in abi.SOILTEMP_FIELDS + abi.SOILWATER_FIELDS}


class ColumnRange:
    """The columns [c0, c1) of a device state, as the drop-in calls see them: column
    pointers advanced by c0 (same ldc), patch and landunit arrays whole."""
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


def copy_segments(handle, pairs, stream):
    """dst <- src for each (dst, src) tensor pair of equal size, through
    clmgb_copy_segments: one kernel per 128 pairs, evict-first loads."""
    pairs = [(d, s) for d, s in pairs if s.numel() > 0]
    for i in range(0, len(pairs), abi.MAX_COPY_SEGMENTS):
        chunk = pairs[i:i + abi.MAX_COPY_SEGMENTS]
        n = len(chunk)
        dst = (C.c_void_p * n)(*[d.data_ptr() for d, _ in chunk])
        src = (C.c_void_p * n)(*[s.data_ptr() for _, s in chunk])
        nb = (C.c_int64 * n)(*[s.numel() * s.element_size() for _, s in chunk])
        api.check(handle.lib.clmgb_copy_segments(dst, src, nb, n, C.c_void_p(stream.cuda_stream)), "copy_segments")


def nbytes(host, names):
    return int(sum(host[k].numel() * host[k].element_size() for k in names if k in host))


class HostStepper:
    """Device mirror `dev` (a device State) of the pinned host tensors `host` (dict
    name -> pinned torch tensor with the same shapes).  step() runs one column step
    with the four drop-in calls and leaves its results in `host`."""

    def __init__(self, handle, host, dev, dtime, cfg=None, snow_method=abi.SNOW_JORDAN1991, chunks=1,
                 readback="dma"):
        import torch
        self.h, self.host, self.dev, self.dtime = handle, host, dev, dtime
        # "dma": one copy-engine transfer per field; "kernel": the temperature outputs
        # come back through clmgb_copy_segments (evict-first loads) while the Richards
        # solve runs.  On GB300 at 262,144 columns "dma" measured 11.9 M column-steps/s
        # end to end and "kernel" 10.2 M: the copy's blocks slow the solve they share
        # the SMs with more than the copy engine's L2 traffic does.
        if readback not in ("kernel", "dma"):
            raise ValueError("readback must be 'kernel' or 'dma'")
        self.readback = readback
        self.cfg = cfg or abi.SwmConfig.clm5_default()
        self.snow_method = snow_method
        for k, v in host.items():         # the whole state once; STATIC stays resident
            dev[k].copy_(v)
        torch.cuda.synchronize()
        self.inputs = [k for k in INPUTS if k in host]
        self.out_t = [k for k in WRITTEN_TEMPERATURE if k in host]
        self.out_w = [k for k in WRITTEN_WATER if k in host]
        self.copy_stream = torch.cuda.Stream()
        self.h2d_bytes = nbytes(host, self.inputs)
        self.d2h_bytes = nbytes(host, self.out_t) + nbytes(host, self.out_w)
        # column ranges, and the patch range of each (patches of consecutive columns
        # must be consecutive for a range's patch fields to move with it)
        nc = dev.nc
        edges = np.linspace(0, nc, max(1, int(chunks)) + 1).astype(np.int64)
        self.ranges = [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]
        pi = host["col_patchi"].numpy()
        pf = host["col_patchf"].numpy()
        self.prange = []
        for (a, b) in self.ranges:
            p0, p1 = int(pi[a:b].min()) - 1, int(pf[a:b].max())
            self.prange.append((p0, max(p0, p1)))
        ok = all(self.prange[i][1] <= self.prange[i + 1][0] for i in range(len(self.prange) - 1))
        if len(self.ranges) > 1 and not ok:
            raise ValueError("chunked steps need the patches of consecutive columns to be consecutive")
        self.in_stream = torch.cuda.Stream()
        self.ldc, self.ldp = dev.bounds().ldc, dev.bounds().ldp

    def _move(self, name, i, to_device, stream):
        """Copy field `name` of range i between host and device on `stream`."""
        h, d = self.host[name], self.dev[name]
        kind = _KIND.get(name, "c")
        if kind == "c":
            a, b = self.ranges[i]
            ld = self.ldc
        elif kind == "p":
            a, b = self.prange[i]
            ld = self.ldp
        else:
            if i == 0 and to_device:
                d.copy_(h, non_blocking=True)
            return
        es = h.element_size()
        rows = h.shape[0] if h.dim() == 2 else 1
        off = a * es
        hp, dp = h.data_ptr() + off, d.data_ptr() + off
        dst, src = (dp, hp) if to_device else (hp, dp)
        api.check(self.h.lib.clmgb_copy_columns(C.c_void_p(dst), ld * es, C.c_void_p(src), ld * es, (b - a) * es,
                                                rows, C.c_void_p(stream.cuda_stream)), "copy_columns")

    def step_chunked(self, stream=None, forcing=None):
        """One step over the column ranges, uploads and read-backs overlapped with the
        other ranges' compute.  forcing(view), when given, runs on each range's
        ColumnRange after its inputs arrive."""
        import torch
        s = stream or torch.cuda.current_stream()
        nr = len(self.ranges)
        self.in_stream.wait_stream(s)                    # the previous step is done with the device state
        self.in_stream.wait_stream(self.copy_stream)     # and with the host arrays
        ev_in = []
        for i in range(nr):
            for k in self.inputs:
                self._move(k, i, True, self.in_stream)
            e = torch.cuda.Event()
            e.record(self.in_stream)
            ev_in.append(e)
        try:
            for i, (a, b) in enumerate(self.ranges):
                view = ColumnRange(self.dev, a, b)
                s.wait_event(ev_in[i])
                self.h.set_option(abi.OPT_COLUMN_BASE, a)
                with torch.cuda.stream(s):
                    if forcing is not None:
                        forcing(view)
                    api.soil_temperature(self.h, view, self.dtime, self.snow_method, stream=s)
                    api.set_soil_water_fractions(self.h, view, stream=s)
                    et = torch.cuda.Event()
                    et.record(s)
                self.copy_stream.wait_event(et)
                for k in self.out_t:
                    self._move(k, i, False, self.copy_stream)
        finally:
            self.h.set_option(abi.OPT_COLUMN_BASE, 0)
        # the Richards solve over all columns at once: its work queue balances the
        # columns' very different substep counts only across many columns per lane
        # (a quarter of 262,144 columns took 12.4 ms against 13.9 ms for all of them)
        with torch.cuda.stream(s):
            api.soil_water(self.h, self.dev, self.dtime, self.cfg, stream=s)
            for k in self.out_w:
                self.host[k].copy_(self.dev[k], non_blocking=True)
        s.wait_stream(self.copy_stream)                  # the step ends when its results are on the host

    def step(self, stream=None, forcing=None):
        """One step on `stream` (default: the current stream).  forcing(dev), when
        given, runs on the device after the inputs arrive (input injection)."""
        import torch
        s = stream or torch.cuda.current_stream()
        dev, host = self.dev, self.host
        with torch.cuda.stream(s):
            for k in self.inputs:
                dev[k].copy_(host[k], non_blocking=True)
            if forcing is not None:
                forcing(dev)
            api.soil_temperature(self.h, dev, self.dtime, self.snow_method, stream=s)
            api.set_soil_water_fractions(self.h, dev, stream=s)
            ev = torch.cuda.Event()
            ev.record(s)
        self.copy_stream.wait_event(ev)
        with torch.cuda.stream(self.copy_stream):
            if self.readback == "kernel":
                copy_segments(self.h, [(host[k], dev[k]) for k in self.out_t], self.copy_stream)
            else:
                for k in self.out_t:
                    host[k].copy_(dev[k], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.copy_stream)
        with torch.cuda.stream(s):
            api.soil_water(self.h, dev, self.dtime, self.cfg, stream=s)
            for k in self.out_w:
                host[k].copy_(dev[k], non_blocking=True)
        s.wait_event(done)        # the next step's inputs must not overtake the read-back
