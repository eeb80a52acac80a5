"""Algorithmic HBM bytes of one column-step (the roofline numerator).

Each field the path must read or write counts once per column-step, 8 bytes per
Float64/Int64 word, active levels only (the frozen field list of the hot path):

soil/bedrock levels (nlevgrnd = 25):
  read   dz, z, zi, watsat, tkmg, tkdry, csol, bsw, sucsat, excess_ice      10
  r+w    t_soisno, h2osoi_liq, h2osoi_ice                                    6
  write  fact, thk, imelt, exice_subs, eflx_fgr                             5
hydrologically active levels (nlevsoi = 20), in addition:
  read   hksat, qflx_rootsoi; write smp_l, hk_l, icefrac, eff_porosity      6
per column: 55 words (patch fluxes, fractions, snow/surface-water state, xmf,
  snowmelt fluxes, t_grnd, qcharge, num_substeps, eflx_fgr12, forcing)
per active snow level: 16 words (read dz, z, zi, sabg_lyr; r+w t, liq, ice;
  write fact, thk, imelt, bw, qflx_snomelt_lyr, qflx_snofrz_lyr)
"""
import numpy as np

SOIL_WORDS_PER_LEVEL = 21
HYDRO_WORDS_PER_LEVEL = 6
COLUMN_WORDS = 55
SNOW_WORDS_PER_LEVEL = 16
WORD = 8


def bytes_per_column_step(nsnow, nlevgrnd=25, nlevsoi=20):
    """Bytes for one column with `nsnow` active snow layers (array-friendly)."""
    words = (SOIL_WORDS_PER_LEVEL * nlevgrnd + HYDRO_WORDS_PER_LEVEL * nlevsoi + COLUMN_WORDS
             + SNOW_WORDS_PER_LEVEL * np.asarray(nsnow))
    return WORD * words


def bytes_per_step(snl, nlevgrnd=25, nlevsoi=20):
    """Total algorithmic bytes of one timestep over all columns (snl <= 0 per column)."""
    nsnow = -np.asarray(snl, dtype=np.int64)
    return int(np.sum(bytes_per_column_step(nsnow, nlevgrnd, nlevsoi)))


# The moisture-form Richards kernel alone (soilwm_moisture_form_solve!), per column:
# per active layer read h2osoi_liq, dz, z, watsat, bsw, sucsat, hksat, qflx_rootsoi,
# icefrac (9 words) and write h2osoi_liq, smp_l, hk_l (3 words); per column mask,
# nbedrock, qflx_infl, qcharge, num_substeps (5 words).
RICHARDS_WORDS_PER_LAYER = 12
RICHARDS_COLUMN_WORDS = 5


def richards_bytes_per_call(nc, nlevsoi=20):
    return int(WORD * nc * (RICHARDS_WORDS_PER_LAYER * nlevsoi + RICHARDS_COLUMN_WORDS))
