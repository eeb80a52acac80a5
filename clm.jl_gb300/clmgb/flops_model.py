"""FP64 work model of the moisture-form Richards solve (the dominant kernel), for the
second roofline of the column solve: on GB300 the FP64 pipe, not HBM, bounds it.

Operations are counted from the kernel source per soil level, separately for a substep
attempt and for a hydraulic refresh (the properties, fluxes and derivatives formed
after every accepted substep, plus that substep's water update):

  attempt (mf_attempt, clmgb_device.cuh; soil_water_movement.jl:1380-1463)
    matrix entries and the Thomas forward sweep: amx 1, bmx 3, cmx 1, rmx 1, the
    recurrence bet 2 and dwat 2, with the divisions gam = cmx/bet and dwat = ../bet;
    back substitution 2; error estimate fnet0 = dwat/dt_dz (a division) and 3 more:
    15 add/mul + 3 divisions per level
  refresh (mfp_refresh, kernels.cu; :1280-1378, :1466-1470)
    saturation: 2 divisions; hydraulic properties: 9 add/mul, 3 divisions and the two
    pow of s^(2b+3) and s^(-b); fluxes and derivatives: 13 add/mul and 5 divisions; net
    flux 2; the accepted substep's water update 3:
    27 add/mul + 10 divisions + 2 pow per level

An add, subtract or multiply is one FP64 pipe instruction, as a DFMA is.  A pow
(clm_math.h, a double-double logarithm and exponential) is a sequence of them; its cost
in DFMA-equivalents is the ratio of the DFMA rate to its rate, both measured on the
device by the probe (clm.jl_gb300/probe/fp64_probe.cu).  The divisions run on the
integer pipes (jl_div: cm_div's 64-bit reciprocal and 2/1 division), not on the FP64
pipe, so they add nothing to the FP64 work; they are counted separately.  The kernel
counts the levels of its attempts and refreshes itself (CLMGB_OPT_COUNT_WORK), so

  DFMA-equivalents = level_attempts * 15 + level_refreshes * (27 + 2 w_pow)
  integer-pipe divisions = level_attempts * 3 + level_refreshes * 10

and the FP64 fraction of a launch is that work over (launch time x measured DFMA rate).
"""

ATTEMPT = {"ops": 15, "div": 3, "pow": 0}
REFRESH = {"ops": 27, "div": 10, "pow": 2}


def weights(probe):
    """DFMA-equivalents of a division and of a pow from the probe's rates
    (dfma_per_s, div_per_s, pow_per_s, log10_per_s)."""
    dfma, div, pw = probe[0], probe[1], probe[2]
    return {"div": dfma / div, "pow": dfma / pw}


def dfma_equivalents(level_attempts, level_refreshes, w):
    """FP64-pipe work; the divisions run on the integer pipes."""
    per_att = ATTEMPT["ops"] + ATTEMPT["pow"] * w["pow"]
    per_ref = REFRESH["ops"] + REFRESH["pow"] * w["pow"]
    return level_attempts * per_att + level_refreshes * per_ref


def integer_divisions(level_attempts, level_refreshes):
    return level_attempts * ATTEMPT["div"] + level_refreshes * REFRESH["div"]


def fp64_roofline(level_attempts, level_refreshes, launches, kernel_ms, probe):
    """The roofline entry of the FP64 pipe for the mean launch."""
    w = weights(probe)
    work = dfma_equivalents(level_attempts, level_refreshes, w) / launches
    achieved = work / (kernel_ms / 1000.0)
    return {"bound": "fp64", "achieved": achieved * 2 / 1e12, "peak": probe[0] * 2 / 1e12,
            "unit": "TFLOP/s (DFMA-equivalent)", "frac": achieved / probe[0],
            "dfma_equivalents_per_launch": work, "level_attempts_per_launch": level_attempts / launches,
            "level_refreshes_per_launch": level_refreshes / launches,
            "integer_pipe_divisions_per_launch": integer_divisions(level_attempts, level_refreshes) / launches,
            "weights_dfma_equivalents": w, "probe_rates_per_s": {"dfma": probe[0], "div": probe[1],
                                                                 "pow": probe[2], "log10": probe[3],
                                                                 "integer_div": probe[4] if len(probe) > 4 else None}}
