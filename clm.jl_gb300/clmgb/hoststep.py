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
  soil_temperature! and set_soil_water_fractions! have run are read back by the copy
  engine on a second stream while the Richards solve runs; the Richards outputs follow
  it.

The arithmetic is the device step's: the host arrays end up bit for bit as a
device-resident run leaves its state (tests/test_gpu_hoststep.py).
"""
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



def nbytes(host, names):
    return int(sum(host[k].numel() * host[k].element_size() for k in names if k in host))


class HostStepper:
    """Device mirror `dev` (a device State) of the pinned host tensors `host` (dict
    name -> pinned torch tensor with the same shapes).  step() runs one column step
    with the four drop-in calls and leaves its results in `host`.

    Measured on GB300 at 262,144 columns and dropped: reading the temperature outputs
    back with a copy kernel instead of the copy engine (its blocks slow the solve they
    share the SMs with), steps over column ranges with the uploads and read-backs
    overlapping the other ranges (launch overhead and tails outweigh the overlap), and
    the kernels storing their outputs straight into the pinned host arrays (stores over
    the host link stall the soil-temperature kernel)."""

    def __init__(self, handle, host, dev, dtime, cfg=None, snow_method=abi.SNOW_JORDAN1991):
        import torch
        self.h, self.host, self.dev, self.dtime = handle, host, dev, dtime
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
            for k in self.out_t:
                host[k].copy_(dev[k], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.copy_stream)
        with torch.cuda.stream(s):
            api.soil_water(self.h, dev, self.dtime, self.cfg, stream=s)
            for k in self.out_w:
                host[k].copy_(dev[k], non_blocking=True)
        s.wait_event(done)        # the next step's inputs must not overtake the read-back
