"""Field-by-field comparison of a GPU result state with the oracle's."""
import numpy as np

FLOAT_OUT = ["t_soisno", "h2osoi_liq", "h2osoi_ice", "t_h2osfc", "t_grnd", "fact", "thk", "xmf", "xmf_h2osfc",
             "c_h2osfc", "eflx_fgr12", "eflx_fgr", "eflx_snomelt", "eflx_snomelt_r", "eflx_h2osfc_to_snow",
             "eflx_gnet", "dgnetdT", "sabg_chk", "excess_ice", "h2osno_no_layers", "h2osfc", "int_snow",
             "snow_depth", "bw", "exice_subs", "snomelt_accum", "qflx_snomelt", "qflx_snofrz", "qflx_snow_drain",
             "qflx_h2osfc_to_ice", "qflx_snomelt_lyr", "qflx_snofrz_lyr", "eff_porosity", "icefrac", "smp_l",
             "hk_l", "qcharge", "num_substeps", "forc_lwrad", "t_ssbef", "t_h2osfc_bef"]
INT_OUT = ["imelt"]


def compare(gpu, ref, rtol=1e-10, atol=1e-12, fields=None):
    """Returns (report dict field -> max rel err, set of bad column indices)."""
    rep, bad = {}, set()
    for k in (fields or FLOAT_OUT):
        a, b = np.asarray(gpu[k]), np.asarray(ref[k])
        both_nan = np.isnan(a) & np.isnan(b)
        err = np.abs(a - b)
        lim = rtol * np.abs(b) + atol
        viol = (err > lim) & ~both_nan
        viol |= np.isnan(a) != np.isnan(b)
        denom = np.maximum(np.abs(b), 1e-300)
        with np.errstate(invalid="ignore"):
            rel = np.where(both_nan, 0.0, err / denom)
        rep[k] = float(np.nanmax(rel)) if rel.size else 0.0
        if viol.any():
            cols = np.nonzero(viol.reshape(-1, viol.shape[-1]).any(axis=0))[0]
            bad.update(int(c) for c in cols)
    for k in INT_OUT:
        a, b = np.asarray(gpu[k]), np.asarray(ref[k])
        viol = a != b
        rep[k] = int(viol.sum())
        if viol.any():
            bad.update(int(c) for c in np.nonzero(viol.reshape(-1, viol.shape[-1]).any(axis=0))[0])
    return rep, bad


def bit_mismatches(gpu, ref, fields):
    """Number of elements per field whose bits differ (NaN payloads and signed zeros
    included) between two states; {} when every field is identical."""
    out = {}
    for k in fields:
        a, b = np.ascontiguousarray(gpu[k]), np.ascontiguousarray(ref[k])
        if a.dtype == np.float64:
            a, b = a.view(np.uint64), b.view(np.uint64)
        n = int(np.count_nonzero(a != b))
        if n:
            out[k] = n
    return out
