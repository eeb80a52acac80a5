"""ctypes mirror of include/clmgb.h and the structure-of-arrays field schema.

The field lists below follow the C structs member by member (tests/test_abi.py
parses the header and checks the order).  Every per-level field is a Julia
column-major ``Matrix{Float64}(nc, nlev)``: element ``(c, jj)`` lives at
``c + (jj-1)*ldc``.  Host arrays therefore have numpy shape ``(nlev, ldc)``
(C order) and device tensors the same shape.

Field kinds (dimension of the leading axis):
  L  = nlevsno + nlevmaxurbgrnd   (t_soisno, dz, z, h2osoi_*, fact, imelt, thk ...)
  LZ = L + 1                      (zi)
  G  = nlevgrnd                   (soil parameters, eflx_fgr, icefrac ...)
  S  = nlevsno                    (bw, qflx_snomelt_lyr ...)
  S1 = nlevsno + 1                (sabg_lyr, patch)
  SOI = nlevsoi                   (qflx_rootsoi)
"""
import ctypes as C
import re

c_double_p = C.POINTER(C.c_double)
c_int64_p = C.POINTER(C.c_int64)
c_uint8_p = C.POINTER(C.c_uint8)
c_uint32_p = C.POINTER(C.c_uint32)

# ---- constants (include/clmgb.h) ----
CLMGB_OK = 0
CLMGB_ERR_NULL_ARG = -1
CLMGB_ERR_DIMS = -2
CLMGB_ERR_CONFIG = -3
CLMGB_ERR_UNSUPPORTED = -4
CLMGB_ERR_CUDA = -5
CLMGB_ERR_ABI = -6
CLMGB_ERR_HANDLE = -7

COL_URBAN = 1
COL_SUBSTEP_CAP = 2
COL_NONFINITE = 4
COL_LEVEL_RANGE = 8
COL_PATCH_RANGE = 16

SNOW_JORDAN1991 = 1
SNOW_STURM1997 = 2

BC_HEAD, BC_FLUX, BC_ZERO_FLUX, BC_WATERTABLE, BC_AQUIFER = 0, 1, 2, 3, 4
ZENGDECKER_2009, MOISTURE_FORM = 0, 1

OPT_STEP_SCHEDULE = 1
SCHEDULE_FUSED = 0
SCHEDULE_QUEUE = 1
SCHEDULE_WAVES = 2
OPT_QUEUE_BLOCKS_PER_SM = 2
OPT_QUEUE_OCCUPANCY = 3
OPT_NUM_SMS = 4
OPT_QUEUE_ORDER = 5
OPT_RESERVED_COLUMNS = 6
OPT_WAVES_BLOCKS_PER_SM = 7
OPT_WAVES_OCCUPANCY = 8
OPT_ADJ_TAPE_USED = 9
OPT_ADJ_TAPE_SLOTS = 10
OPT_ADJ_TAPE_ENTRIES = 11
OPT_ADJ_RICHARDS = 12
ADJ_RICHARDS_CLOSED_FORM, ADJ_RICHARDS_RECORDED = 0, 1
OPT_ADJ_SOIL_TEMPERATURE = 13
ADJ_ST_CLOSED_FORM, ADJ_ST_RECORDED = 0, 1
OPT_QUEUE_FRESH_BATCH = 14
OPT_COLUMN_BASE = 15
OPT_QUEUE_DEFER = 16
OPT_QUEUE_PACKED_REFRESH = 17
OPT_ATTEMPT_CAP = 18
OPT_QUEUE_POLL_LIMIT = 19
OPT_QUEUE_PUBLISH_DELAY = 20
OPT_COUNT_WORK = 21
OPT_WORK_LEVEL_ATTEMPTS = 22
OPT_WORK_LEVEL_REFRESHES = 23
OPT_RECORDS_TMA = 24
OPT_RECORDS_TMA_USED = 25
OPT_TRIDIAG_METHOD = 26
OPT_ST_BLOCK = 27
TRIDIAG_THOMAS, TRIDIAG_PCR = 0, 1

COL_URBAN, COL_SUBSTEP_CAP, COL_NONFINITE, COL_LEVEL_RANGE, COL_PATCH_RANGE = 1, 2, 4, 8, 16
COL_ADJ_UNSUPPORTED, COL_TAPE_FULL, COL_ADJ_REPLAY, COL_FILTER, COL_QUEUE_WAIT = 32, 64, 128, 256, 512
COL_COPY_WAIT = 1024
ADJ_MAX_SUBSTEPS = 128

CLMGB_NOALLOC_MAX_COLUMNS = 1 << 20

MAX_NLEVSNO = 12
MAX_NLEVGRND = 25
MAX_NLEVSOI = 25
LOG_REC = MAX_NLEVSOI + 2
LOG_FIN = 3 * MAX_NLEVSOI + 3


LOG_ST_STRIDE = 464        # doubles of a column's soil_temperature! record


def log_stride(cap):
    """Doubles per column of a substep log with `cap` records (CLMGB_LOG_STRIDE)."""
    return cap * LOG_REC + LOG_FIN


class Varpar(C.Structure):
    _fields_ = [("nlevsno", C.c_int32), ("nlevgrnd", C.c_int32), ("nlevsoi", C.c_int32),
                ("nlevurb", C.c_int32), ("nlevmaxurbgrnd", C.c_int32), ("reserved", C.c_int32)]


class Bounds(C.Structure):
    _fields_ = [("nc", C.c_int64), ("np", C.c_int64), ("nl", C.c_int64),
                ("ldc", C.c_int64), ("ldp", C.c_int64)]


class SwmConfig(C.Structure):
    """SoilWaterMovementConfig (soil_water_movement.jl:654-671)."""
    _fields_ = [("soilwater_movement_method", C.c_int32), ("upper_boundary_condition", C.c_int32),
                ("lower_boundary_condition", C.c_int32), ("flux_calculation", C.c_int32),
                ("dtmin", C.c_double), ("verySmall", C.c_double), ("xTolerUpper", C.c_double),
                ("xTolerLower", C.c_double), ("e_ice", C.c_double)]

    @classmethod
    def clm5_default(cls):
        """The config clm_drv! builds when use_aquifer_layer=false (clm_driver.jl:2043-2048)."""
        return cls(MOISTURE_FORM, BC_FLUX, BC_ZERO_FLUX, 1, 60.0, 1.0e-8, 1.0e-1, 1.0e-2, 6.0)


# clmgb_surface_hydrology stages (CLMGB_SH_*), in the driver's order
SH_FLOODC, SH_SAT_EXCESS, SH_QFLX_INPUTS, SH_INFL_EXCESS, SH_ROUTE = 1, 2, 4, 8, 16
SH_UPDATE_H2OSFC, SH_INFILTRATION, SH_TOTAL_RUNOFF, SH_URBAN_PONDING = 32, 64, 128, 256
SH_ALL = 511
FSAT_TOPMODEL, FSAT_VIC = 1, 2
QINMAX_NONE, QINMAX_HKSAT = 0, 1


class SurfHydConfig(C.Structure):
    """clmgb_surfhyd_config: the parameters, method flags and keyword arguments of the
    surface-hydrology routines."""
    _fields_ = [("struct_size", C.c_int64), ("ng", C.c_int64), ("fsat_method", C.c_int32),
                ("crop_fsat_equals_zero", C.c_int32), ("hillslope_fsat_equals_zero", C.c_int32),
                ("qinmax_method", C.c_int32), ("h2osfcflag", C.c_int32), ("update_h2osfcflag", C.c_int32),
                ("fff", C.c_double), ("e_ice", C.c_double), ("pc", C.c_double), ("mu", C.c_double),
                ("pondmx_urban", C.c_double)]

    @classmethod
    def default(cls, ng=1, fff=0.5):
        """TOPModel fsat, hksat qinmax, h2osfcflag 1 (clm_initialize.jl:132-134), e_ice 6
        (infilt_excess_runoff.jl:26), pc 0.4 and mu 0.13889 (surface_water.jl:20-21),
        pondmx_urban 1 mm (varcon.jl:68); fff is read from the parameter file by the
        reference (read_params.jl:23) and is the caller's."""
        return cls(C.sizeof(cls), ng, FSAT_TOPMODEL, 0, 0, QINMAX_HKSAT, 1, 1, fff, 6.0, 0.4, 0.13889, 1.0)


# clmgb_snow_layers stages (CLMGB_SL_*), in the driver's order
SL_COMPACTION, SL_COMBINE, SL_DIVIDE, SL_ZERO_EMPTY, SL_FILTER, SL_ALL = 1, 2, 4, 8, 16, 31
OVERBURDEN_ANDERSON1976, OVERBURDEN_VIONNET2012 = 1, 2


class SnowLayerConfig(C.Structure):
    """clmgb_snowlayer_config: SnowHydrologyParams and the snow module switches."""
    _fields_ = [("struct_size", C.c_int64), ("ng", C.c_int64), ("use_subgrid_fluxes", C.c_int32),
                ("overburden_method", C.c_int32), ("wind_dependent_snow_density", C.c_int32),
                ("is_lake", C.c_int32)] + [(n, C.c_double) for n in (
                    "int_snow_max", "overburden_compress_tfactor", "upplim_destruct_metamorph", "eta0_anderson",
                    "eta0_vionnet", "ceta", "drift_gs", "rho_min", "rho_max", "tau_ref", "snw_rds_min",
                    "snw_rds_max", "dzmin_1", "dzmin_2", "dzmax_l_1", "dzmax_l_2", "dzmax_u_1", "dzmax_u_2")]

    @classmethod
    def default(cls, ng=1):
        """The reference's defaults (snow_hydrology.jl:43-63, 90-101; varctl.jl:79;
        SNW_RDS_MAX, snow_snicar.jl:35; int_snow_max 2000 mm, clm_driver.jl:2154)."""
        return cls(C.sizeof(cls), ng, 1, OVERBURDEN_ANDERSON1976, 0, 0, 2000.0, 0.08, 100.0, 9.0e5, 7.62237e6, 250.0,
                   0.35, 50.0, 350.0, 172800.0, 54.526, 1500.0, 0.010, 0.015, 0.03, 0.07, 0.02, 0.05)


BAL_H2O_WARN, BAL_H2O_ERROR, BAL_H2O_NONFINITE, BAL_SOI_WARN, BAL_SOI_ERROR = 1, 2, 4, 8, 16


class BalanceReport(C.Structure):
    """clmgb_balance_report."""
    _fields_ = [("errh2o_max", C.c_double), ("errh2o_index", C.c_int64), ("errh2o_nonfinite", C.c_int64),
                ("errsoi_max", C.c_double), ("errsoi_index", C.c_int64), ("flags", C.c_uint32),
                ("reserved", C.c_uint32)]


NLEVLAK = 10                      # varpar.nlevlak
MAX_NLEVLAK = 16


class LakeConfig(C.Structure):
    """clmgb_lake_config: varpar.nlevlak and the lake_con sub-options."""
    _fields_ = [("struct_size", C.c_int64), ("nlevlak", C.c_int32), ("use_lch4", C.c_int32),
                ("lakepuddling", C.c_int32), ("lake_no_ed", C.c_int32), ("deepmixing_depthcrit", C.c_double),
                ("deepmixing_mixfact", C.c_double), ("lake_puddle_thick", C.c_double)]

    @classmethod
    def default(cls):
        """nlevlak 10, no CH4, lake_con defaults (lake_temperature.jl:15-23)."""
        return cls(C.sizeof(cls), NLEVLAK, 0, 0, 0, 25.0, 10.0, 0.2)


# (name, ctype, kind, dims) ; kind: 'c' column, 'p' patch, 'l' landunit
# dims: None = vector, else level-kind string
_u8, _i64, _f64 = "u8", "i64", "f64"

SOILTEMP_FIELDS = [
    ("mask_nolakec", _u8, "c", None),
    ("mask_nolakep", _u8, "p", None),
    ("col_snl", _i64, "c", None),
    ("col_nbedrock", _i64, "c", None),
    ("col_itype", _i64, "c", None),
    ("col_landunit", _i64, "c", None),
    ("col_patchi", _i64, "c", None),
    ("col_patchf", _i64, "c", None),
    ("lun_itype", _i64, "l", None),
    ("lun_urbpoi", _u8, "l", None),
    ("patch_column", _i64, "p", None),
    ("patch_landunit", _i64, "p", None),
    ("patch_wtcol", _f64, "p", None),
    ("frac_veg_nosno", _i64, "p", None),
    ("dz", _f64, "c", "L"),
    ("z", _f64, "c", "L"),
    ("zi", _f64, "c", "LZ"),
    ("t_soisno", _f64, "c", "L"),
    ("t_h2osfc", _f64, "c", None),
    ("t_grnd", _f64, "c", None),
    ("xmf", _f64, "c", None),
    ("xmf_h2osfc", _f64, "c", None),
    ("fact", _f64, "c", "L"),
    ("c_h2osfc", _f64, "c", None),
    ("imelt", _i64, "c", "L"),
    ("emg", _f64, "c", None),
    ("htvp", _f64, "c", None),
    ("eflx_bot", _f64, "c", None),
    ("eflx_fgr12", _f64, "c", None),
    ("eflx_fgr", _f64, "c", "G"),
    ("eflx_snomelt", _f64, "c", None),
    ("eflx_snomelt_r", _f64, "c", None),
    ("eflx_snomelt_u", _f64, "c", None),
    ("eflx_h2osfc_to_snow", _f64, "c", None),
    ("eflx_gnet", _f64, "p", None),
    ("dgnetdT", _f64, "p", None),
    ("dlrad", _f64, "p", None),
    ("cgrnd", _f64, "p", None),
    ("eflx_sh_grnd", _f64, "p", None),
    ("eflx_sh_snow", _f64, "p", None),
    ("eflx_sh_soil", _f64, "p", None),
    ("eflx_sh_h2osfc", _f64, "p", None),
    ("watsat", _f64, "c", "G"),
    ("bsw", _f64, "c", "G"),
    ("sucsat", _f64, "c", "G"),
    ("tkmg", _f64, "c", "G"),
    ("tkdry", _f64, "c", "G"),
    ("csol", _f64, "c", "G"),
    ("thk", _f64, "c", "L"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("excess_ice", _f64, "c", "L"),
    ("h2osno_no_layers", _f64, "c", None),
    ("h2osfc", _f64, "c", None),
    ("int_snow", _f64, "c", None),
    ("frac_sno_eff", _f64, "c", None),
    ("frac_h2osfc", _f64, "c", None),
    ("snow_depth", _f64, "c", None),
    ("bw", _f64, "c", "S"),
    ("exice_subs", _f64, "c", "G"),
    ("snomelt_accum", _f64, "c", None),
    ("qflx_evap_soi", _f64, "p", None),
    ("qflx_ev_snow", _f64, "p", None),
    ("qflx_ev_soil", _f64, "p", None),
    ("qflx_ev_h2osfc", _f64, "p", None),
    ("qflx_snomelt", _f64, "c", None),
    ("qflx_snofrz", _f64, "c", None),
    ("qflx_snow_drain", _f64, "c", None),
    ("qflx_h2osfc_to_ice", _f64, "c", None),
    ("qflx_snomelt_lyr", _f64, "c", "S"),
    ("qflx_snofrz_lyr", _f64, "c", "S"),
    ("sabg", _f64, "p", None),
    ("sabg_soil", _f64, "p", None),
    ("sabg_snow", _f64, "p", None),
    ("sabg_lyr", _f64, "p", "S1"),
    ("sabg_chk", _f64, "p", None),
    ("forc_lwrad", _f64, "c", None),
]

SOILWATER_FIELDS = [
    ("mask_hydrology", _u8, "c", None),
    ("col_nbedrock", _i64, "c", None),
    ("dz", _f64, "c", "L"),
    ("z", _f64, "c", "L"),
    ("zi", _f64, "c", "LZ"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("excess_ice", _f64, "c", "L"),
    ("watsat", _f64, "c", "G"),
    ("hksat", _f64, "c", "G"),
    ("bsw", _f64, "c", "G"),
    ("sucsat", _f64, "c", "G"),
    ("eff_porosity", _f64, "c", "G"),
    ("icefrac", _f64, "c", "G"),
    ("smp_l", _f64, "c", "G"),
    ("hk_l", _f64, "c", "G"),
    ("qflx_rootsoi", _f64, "c", "SOI"),
    ("qflx_infl", _f64, "c", None),
    ("zwt", _f64, "c", None),
    ("qcharge", _f64, "c", None),
    ("num_substeps", _f64, "c", None),
    ("smpmin", _f64, "c", None),
]

# clmgb_rootsink_fields (compute_effec_rootfrac_and_vert_tran_sink!), header order;
# HYDRSTRESS_ONLY may be NULL for the default method
ROOTSINK_FIELDS = [
    ("mask_hydrology", _u8, "c", None),
    ("col_itype", _i64, "c", None),
    ("col_landunit", _i64, "c", None),
    ("lun_itype", _i64, "l", None),
    ("col_patchi", _i64, "c", None),
    ("col_npatches", _i64, "c", None),
    ("patch_active", _u8, "p", None),
    ("patch_wtcol", _f64, "p", None),
    ("rootr_patch", _f64, "p", "G"),
    ("qflx_tran_veg_patch", _f64, "p", None),
    ("qflx_tran_veg_col", _f64, "c", None),
    ("rootr_col", _f64, "c", "G"),
    ("qflx_rootsoi_col", _f64, "c", "SOI"),
    ("k_soil_root_patch", _f64, "p", "SOI"),
    ("smp_l", _f64, "c", "G"),
    ("vegwp_patch", _f64, "p", "V4"),
    ("frac_veg_nosno", _i64, "p", None),
    ("z", _f64, "c", "L"),
    ("qflx_phs_neg_col", _f64, "c", None),
    ("qflx_hydr_redist_patch", _f64, "p", None),
]
# clmgb_soilflux_fields (soil_fluxes!), header order
SOILFLUX_FIELDS = [
    ("mask_nolakec", _u8, "c", None),
    ("mask_nolakep", _u8, "p", None),
    ("mask_urbanp", _u8, "p", None),
    ("col_snl", _i64, "c", None),
    ("col_itype", _i64, "c", None),
    ("col_patchi", _i64, "c", None),
    ("col_patchf", _i64, "c", None),
    ("lun_itype", _i64, "l", None),
    ("lun_urbpoi", _u8, "l", None),
    ("patch_column", _i64, "p", None),
    ("patch_landunit", _i64, "p", None),
    ("patch_wtcol", _f64, "p", None),
    ("frac_veg_nosno", _i64, "p", None),
    ("frac_sno_eff", _f64, "c", None),
    ("frac_h2osfc", _f64, "c", None),
    ("t_ssbef", _f64, "c", "L"),
    ("t_h2osfc_bef", _f64, "c", None),
    ("t_grnd", _f64, "c", None),
    ("t_h2osfc", _f64, "c", None),
    ("emg", _f64, "c", None),
    ("t_soisno", _f64, "c", "L"),
    ("fact", _f64, "c", "L"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("htvp", _f64, "c", None),
    ("xmf", _f64, "c", None),
    ("xmf_h2osfc", _f64, "c", None),
    ("c_h2osfc", _f64, "c", None),
    ("eflx_h2osfc_to_snow", _f64, "c", None),
    ("eflx_building_heat_errsoi", _f64, "c", None),
    ("forc_lwrad", _f64, "c", None),
    ("errsoi_col", _f64, "c", None),
    ("cgrnds", _f64, "p", None),
    ("cgrndl", _f64, "p", None),
    ("sabg", _f64, "p", None),
    ("sabg_soil", _f64, "p", None),
    ("sabg_snow", _f64, "p", None),
    ("dlrad", _f64, "p", None),
    ("ulrad", _f64, "p", None),
    ("eflx_sh_veg", _f64, "p", None),
    ("eflx_sh_stem", _f64, "p", None),
    ("eflx_wasteheat", _f64, "p", None),
    ("eflx_heat_from_ac", _f64, "p", None),
    ("eflx_traffic", _f64, "p", None),
    ("eflx_ventilation", _f64, "p", None),
    ("qflx_evap_veg", _f64, "p", None),
    ("qflx_tran_veg", _f64, "p", None),
    ("eflx_sh_grnd", _f64, "p", None),
    ("qflx_evap_soi", _f64, "p", None),
    ("qflx_ev_soil", _f64, "p", None),
    ("qflx_ev_h2osfc", _f64, "p", None),
    ("qflx_ev_snow", _f64, "p", None),
    ("eflx_lwrad_net", _f64, "p", None),
    ("eflx_lwrad_out", _f64, "p", None),
    ("eflx_lwrad_net_u", _f64, "p", None),
    ("eflx_sh_tot", _f64, "p", None),
    ("eflx_sh_tot_r", _f64, "p", None),
    ("eflx_sh_tot_u", _f64, "p", None),
    ("eflx_lh_tot", _f64, "p", None),
    ("eflx_lh_tot_r", _f64, "p", None),
    ("eflx_lh_tot_u", _f64, "p", None),
    ("eflx_lh_vege", _f64, "p", None),
    ("eflx_lh_vegt", _f64, "p", None),
    ("eflx_lh_grnd", _f64, "p", None),
    ("eflx_soil_grnd", _f64, "p", None),
    ("eflx_soil_grnd_r", _f64, "p", None),
    ("eflx_soil_grnd_u", _f64, "p", None),
    ("eflx_lwrad_net_r", _f64, "p", None),
    ("eflx_lwrad_out_r", _f64, "p", None),
    ("eflx_lwrad_out_u", _f64, "p", None),
    ("errsoi_patch", _f64, "p", None),
    ("t_skin", _f64, "p", None),
    ("qflx_evap_tot", _f64, "p", None),
    ("qflx_evap_can", _f64, "p", None),
    ("qflx_liqevap_from_top_layer", _f64, "p", None),
    ("qflx_solidevap_from_top_layer", _f64, "p", None),
    ("qflx_soliddew_to_top_layer", _f64, "p", None),
    ("qflx_liqdew_to_top_layer", _f64, "p", None),
]

# clmgb_surfhyd_fields (the surface hydrology before soil_water!), header order;
# kind 'g' = gridcell
SURFHYD_FIELDS = [
    ("mask_nolakec", _u8, "c", None),
    ("mask_hydrology", _u8, "c", None),
    ("mask_urban", _u8, "c", None),
    ("col_snl", _i64, "c", None),
    ("col_itype", _i64, "c", None),
    ("col_landunit", _i64, "c", None),
    ("col_gridcell", _i64, "c", None),
    ("col_urbpoi", _u8, "c", None),
    ("col_is_hillslope", _u8, "c", None),
    ("col_active", _u8, "c", None),
    ("col_cold", _i64, "c", None),
    ("lun_itype", _i64, "l", None),
    ("qflx_floodg", _f64, "g", None),
    ("frost_table", _f64, "c", None),
    ("zwt", _f64, "c", None),
    ("zwt_perched", _f64, "c", None),
    ("wtfact", _f64, "c", None),
    ("b_infil", _f64, "c", None),
    ("top_max_moist", _f64, "c", None),
    ("top_moist_limited", _f64, "c", None),
    ("icefrac", _f64, "c", "G"),
    ("hksat", _f64, "c", "G"),
    ("frac_sno_eff", _f64, "c", None),
    ("frac_h2osfc", _f64, "c", None),
    ("frac_h2osfc_nosnow", _f64, "c", None),
    ("h2osfc_thresh", _f64, "c", None),
    ("topo_slope", _f64, "c", None),
    ("qflx_rain_plus_snomelt", _f64, "c", None),
    ("qflx_snow_h2osfc", _f64, "c", None),
    ("qflx_liqevap_from_top_layer", _f64, "c", None),
    ("qflx_ev_soil", _f64, "c", None),
    ("qflx_ev_h2osfc", _f64, "c", None),
    ("qflx_floodc", _f64, "c", None),
    ("fsat", _f64, "c", None),
    ("fcov", _f64, "c", None),
    ("qflx_sat_excess_surf", _f64, "c", None),
    ("qflx_top_soil", _f64, "c", None),
    ("qflx_in_soil", _f64, "c", None),
    ("qflx_top_soil_to_h2osfc", _f64, "c", None),
    ("qinmax", _f64, "c", None),
    ("qflx_infl_excess", _f64, "c", None),
    ("qflx_in_soil_limited", _f64, "c", None),
    ("qflx_in_h2osfc", _f64, "c", None),
    ("qflx_infl_excess_surf", _f64, "c", None),
    ("h2osfc", _f64, "c", None),
    ("qflx_h2osfc_surf", _f64, "c", None),
    ("qflx_h2osfc_drain", _f64, "c", None),
    ("qflx_infl", _f64, "c", None),
    ("qflx_surf", _f64, "c", None),
    ("xs_urban", _f64, "c", None),
    ("h2osoi_liq", _f64, "c", "L"),
]

# clmgb_snowlayer_fields (snow layer dynamics after the soil solve), header order
SNOWLAYER_FIELDS = [
    ("mask_snow", _u8, "c", None),
    ("mask_nosnow", _u8, "c", None),
    ("mask_nolakec", _u8, "c", None),
    ("col_snl", _i64, "c", None),
    ("col_landunit", _i64, "c", None),
    ("col_gridcell", _i64, "c", None),
    ("lun_itype", _i64, "l", None),
    ("lun_lakpoi", _u8, "l", None),
    ("lun_urbpoi", _u8, "l", None),
    ("forc_wind", _f64, "g", None),
    ("n_melt", _f64, "c", None),
    ("frac_h2osfc", _f64, "c", None),
    ("frac_sno", _f64, "c", None),
    ("frac_sno_eff", _f64, "c", None),
    ("int_snow", _f64, "c", None),
    ("h2osno_no_layers", _f64, "c", None),
    ("snow_depth", _f64, "c", None),
    ("qflx_sl_top_soil", _f64, "c", None),
    ("dz", _f64, "c", "L"),
    ("z", _f64, "c", "L"),
    ("zi", _f64, "c", "LZ"),
    ("t_soisno", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("imelt", _i64, "c", "S"),
    ("swe_old", _f64, "c", "S"),
    ("frac_iceold", _f64, "c", "S"),
    ("snw_rds", _f64, "c", "S"),
    ("mss_bcphi", _f64, "c", "S"),
    ("mss_bcpho", _f64, "c", "S"),
    ("mss_ocphi", _f64, "c", "S"),
    ("mss_ocpho", _f64, "c", "S"),
    ("mss_dst1", _f64, "c", "S"),
    ("mss_dst2", _f64, "c", "S"),
    ("mss_dst3", _f64, "c", "S"),
    ("mss_dst4", _f64, "c", "S"),
]

# clmgb_lake_fields (lake_temperature!), header order; level kind "K" = nlevlak
LAKE_FIELDS = [
    ("mask_lakec", _u8, "c", None),
    ("mask_lakep", _u8, "p", None),
    ("col_patchi", _i64, "c", None),
    ("patch_column", _i64, "p", None),
    ("col_snl", _i64, "c", None),
    ("dz", _f64, "c", "L"),
    ("z", _f64, "c", "L"),
    ("zi", _f64, "c", "LZ"),
    ("dz_lake", _f64, "c", "K"),
    ("z_lake", _f64, "c", "K"),
    ("lakedepth", _f64, "c", None),
    ("watsat", _f64, "c", "G"),
    ("tksatu", _f64, "c", "G"),
    ("tkmg", _f64, "c", "G"),
    ("tkdry", _f64, "c", "G"),
    ("csol", _f64, "c", "G"),
    ("t_grnd", _f64, "c", None),
    ("etal", _f64, "c", None),
    ("ks", _f64, "c", None),
    ("ws", _f64, "c", None),
    ("lake_raw", _f64, "c", None),
    ("t_soisno", _f64, "c", "L"),
    ("t_lake", _f64, "c", "K"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("h2osno_no_layers", _f64, "c", None),
    ("snow_depth", _f64, "c", None),
    ("frac_iceold", _f64, "c", "S"),
    ("betaprime", _f64, "c", None),
    ("lake_icefrac", _f64, "c", "K"),
    ("lake_icefracsurf", _f64, "c", None),
    ("lake_icethick", _f64, "c", None),
    ("savedtke1", _f64, "c", None),
    ("lakeresist", _f64, "c", None),
    ("grnd_ch4_cond", _f64, "c", None),
    ("qflx_snomelt", _f64, "c", None),
    ("qflx_snofrz", _f64, "c", None),
    ("qflx_snow_drain", _f64, "c", None),
    ("qflx_snomelt_lyr", _f64, "c", "S"),
    ("qflx_snofrz_lyr", _f64, "c", "S"),
    ("imelt", _i64, "c", "S"),
    ("eflx_snomelt", _f64, "c", None),
    ("errsoi_col", _f64, "c", None),
    ("sabg", _f64, "p", None),
    ("sabg_lyr", _f64, "p", "S1"),
    ("fsds_nir_d", _f64, "p", None),
    ("fsds_nir_i", _f64, "p", None),
    ("fsr_nir_d", _f64, "p", None),
    ("fsr_nir_i", _f64, "p", None),
    ("eflx_gnet", _f64, "p", None),
    ("eflx_sh_tot", _f64, "p", None),
    ("eflx_sh_grnd", _f64, "p", None),
    ("eflx_soil_grnd", _f64, "p", None),
]

# clmgb_colbalance_fields (balance_check!'s column checks), header order
COLBALANCE_FIELDS = [
    ("col_itype", _i64, "c", None),
    ("col_active", _u8, "c", None),
    ("forc_rain", _f64, "c", None),
    ("forc_snow", _f64, "c", None),
    ("begwb", _f64, "c", None),
    ("endwb", _f64, "c", None),
    ("qflx_flood", _f64, "c", None),
    ("qflx_sfc_irrig", _f64, "c", None),
    ("qflx_glcice_dyn_water_flux", _f64, "c", None),
    ("qflx_evap_tot", _f64, "c", None),
    ("qflx_surf", _f64, "c", None),
    ("qflx_qrgwl", _f64, "c", None),
    ("qflx_drain", _f64, "c", None),
    ("qflx_drain_perched", _f64, "c", None),
    ("qflx_ice_runoff", _f64, "c", None),
    ("qflx_snwcp_discarded_liq", _f64, "c", None),
    ("qflx_snwcp_discarded_ice", _f64, "c", None),
    ("errsoi", _f64, "c", None),
    ("errh2o", _f64, "c", None),
]

# clmgb_zd09_fields (soilwater_zengdecker2009!), header order
ZD09_FIELDS = [
    ("mask_hydrology", _u8, "c", None),
    ("dz", _f64, "c", "L"),
    ("z", _f64, "c", "L"),
    ("zi", _f64, "c", "LZ"),
    ("t_soisno", _f64, "c", "L"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("h2osoi_vol", _f64, "c", "G"),
    ("watsat", _f64, "c", "G"),
    ("hksat", _f64, "c", "G"),
    ("bsw", _f64, "c", "G"),
    ("sucsat", _f64, "c", "G"),
    ("smpmin", _f64, "c", None),
    ("icefrac", _f64, "c", "G"),
    ("smp_l", _f64, "c", "G"),
    ("hk_l", _f64, "c", "G"),
    ("qflx_rootsoi", _f64, "c", "SOI"),
    ("qflx_infl", _f64, "c", None),
    ("zwt", _f64, "c", None),
    ("qcharge", _f64, "c", None),
    ("qflx_deficit", _f64, "c", None),
]
HYDRSTRESS_ONLY = ("k_soil_root_patch", "smp_l", "vegwp_patch", "frac_veg_nosno", "z", "qflx_phs_neg_col",
                   "qflx_hydr_redist_patch")

# Fields of the synthetic step harness that are not in either struct.
# clmgb_flexcn_fields (soil_water!'s use_flexibleCN step), header order
FLEXCN_FIELDS = [
    ("mask_hydrology", _u8, "c", None),
    ("dz", _f64, "c", "L"),
    ("h2osoi_liq", _f64, "c", "L"),
    ("h2osoi_ice", _f64, "c", "L"),
    ("h2osoi_vol", _f64, "c", "G"),
    ("wa", _f64, "c", None),
]

EXTRA_FIELDS = [
    ("t_ssbef", _f64, "c", "L"),
    ("t_h2osfc_bef", _f64, "c", None),
]

_CT = {_u8: c_uint8_p, _i64: c_int64_p, _f64: c_double_p}


def _mk_struct(name, fields):
    return type(name, (C.Structure,),
                {"_fields_": [("struct_size", C.c_int64)] + [(n, _CT[t]) for (n, t, _, _) in fields]})


SoilTempFields = _mk_struct("SoilTempFields", SOILTEMP_FIELDS)

# clmgb_step_adjoint: (member, level kind or None for [nc]) in header order
STEP_ADJOINT_MEMBERS = [("lam_t_soisno", "L"), ("lam_h2osoi_liq", "L"), ("lam_h2osoi_ice", "L"),
                        ("lam_t_grnd", None), ("lam_t_h2osfc", None), ("lam_qcharge", None),
                        ("grad_watsat", "SOI"), ("grad_bsw", "SOI"), ("grad_sucsat", "SOI"),
                        ("grad_hksat", "SOI"), ("lam_forc_lwrad", None)]
StepAdjoint = type("StepAdjoint", (C.Structure,),
                   {"_fields_": [("struct_size", C.c_int64)] + [(n, c_double_p) for n, _ in STEP_ADJOINT_MEMBERS]})
SoilWaterFields = _mk_struct("SoilWaterFields", SOILWATER_FIELDS)
RootSinkFields = _mk_struct("RootSinkFields", ROOTSINK_FIELDS)
Zd09Fields = _mk_struct("Zd09Fields", ZD09_FIELDS)
SurfHydFields = _mk_struct("SurfHydFields", SURFHYD_FIELDS)
SnowLayerFields = _mk_struct("SnowLayerFields", SNOWLAYER_FIELDS)
LakeFields = _mk_struct("LakeFields", LAKE_FIELDS)
ColBalanceFields = _mk_struct("ColBalanceFields", COLBALANCE_FIELDS)
SoilFluxFields = _mk_struct("SoilFluxFields", SOILFLUX_FIELDS)
FlexCnFields = _mk_struct("FlexCnFields", FLEXCN_FIELDS)


class SubstepLog(C.Structure):
    """clmgb_substep_log."""
    _fields_ = [("struct_size", C.c_int64), ("rec", c_double_p), ("count", C.POINTER(C.c_int32)),
                ("cap", C.c_int32), ("st_rec", c_double_p)]


def all_fields():
    """Union of every field (first definition wins), in a stable order."""
    seen, out = set(), []
    for fl in (SOILTEMP_FIELDS, SOILWATER_FIELDS, EXTRA_FIELDS):
        for f in fl:
            if f[0] not in seen:
                seen.add(f[0])
                out.append(f)
    return out


def level_count(kind, vp):
    """Number of levels of a field kind for a Varpar-like object."""
    L = vp.nlevsno + vp.nlevmaxurbgrnd
    return {"L": L, "LZ": L + 1, "G": vp.nlevgrnd, "S": vp.nlevsno,
            "S1": vp.nlevsno + 1, "SOI": vp.nlevsoi, "V4": 4, "K": NLEVLAK}[kind]


def header_struct_members(header_text, struct_name):
    """Member names of `typedef struct <struct_name> {...}` in the C header."""
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (struct_name, struct_name), header_text, re.S)
    if not m:
        raise ValueError("struct %s not found" % struct_name)
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        names.append(re.findall(r"([A-Za-z_][A-Za-z0-9_]*)\s*$", decl)[0])
    return names
