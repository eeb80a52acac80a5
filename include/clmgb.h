/*
 * clmgb.h — C ABI of the GB300-native soil/snow column solve.
 *
 * Drop-in boundary for CLM.jl's per-column vertical solve:
 *   soil_temperature!      src/biogeophys/soil_temperature.jl:358-593
 *   set_soil_water_fractions! src/biogeophys/soil_hydrology.jl:394-416 (kernel :110-130)
 *   soil_water! -> soilwater_moisture_form! -> soilwm_moisture_form_solve!
 *                          src/biogeophys/soil_water_movement.jl:1780-1810, 1532-1601, 1498-1517
 *   batched_band_solve!    src/infrastructure/band_diagonal.jl:179-189
 *   tridiagonal_multi!     src/infrastructure/tridiagonal.jl:129-142
 *
 * Layout contract (identical to the reference's structure-of-arrays state):
 *   every per-column level field is a Julia column-major Matrix{Float64}(nc, nlev):
 *   element (c, jj) — c = 0..nc-1, jj = 1..nlev the Julia level index — lives at
 *   ptr[c + (jj-1)*ldc].  ldc >= nc (ldc == nc for a plain Julia Matrix).  Patch
 *   matrices use ldp the same way.  Integer state (snl, nbedrock, imelt, itype,
 *   landunit, patchi/patchf, ...) is int64_t (Julia Int), Bool masks are uint8_t,
 *   and every index stored in an array is 1-based as in Julia.
 *
 * All compute entry points are stream-ordered and asynchronous: they enqueue work on
 * `stream` (a cudaStream_t passed as void*; NULL = legacy default stream) and return.
 * Pointers are device pointers unless stated otherwise.  The library never allocates
 * inside a compute call: scratch lives in the handle (clmgb_create).  A handle is not
 * thread-safe; use one handle per stream.
 *
 * Return codes: 0 success; negative = invalid argument / unsupported configuration
 * detected on the host before any launch (nothing was enqueued); the device-side
 * per-column status (CLMGB_COL_*) is accumulated in the handle and read with
 * clmgb_device_status().  There is no CPU fallback anywhere behind this ABI.
 */
#ifndef CLMGB_H
#define CLMGB_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLMGB_ABI_VERSION 1

/* ---- return codes ---- */
#define CLMGB_OK                 0
#define CLMGB_ERR_NULL_ARG      -1   /* a required pointer is NULL */
#define CLMGB_ERR_DIMS          -2   /* level counts / nc / leading dims out of the supported range */
#define CLMGB_ERR_CONFIG        -3   /* method / boundary condition the reference rejects with error() */
#define CLMGB_ERR_UNSUPPORTED   -4   /* a configuration this build does not implement (no fallback) */
#define CLMGB_ERR_CUDA          -5   /* a CUDA launch or copy failed; see clmgb_last_cuda_error */
#define CLMGB_ERR_ABI           -6   /* struct size / ABI version mismatch */
#define CLMGB_ERR_HANDLE        -7   /* NULL or foreign handle */

/* ---- per-column device status bits (OR-accumulated in the handle) ---- */
#define CLMGB_COL_URBAN          1u  /* urban landunit column reached a non-urban kernel */
#define CLMGB_COL_SUBSTEP_CAP    2u  /* Richards substep attempts hit the safety cap */
#define CLMGB_COL_NONFINITE      4u  /* a non-finite temperature / water value was produced */
#define CLMGB_COL_LEVEL_RANGE    8u  /* snl / nbedrock outside the level range */
#define CLMGB_COL_PATCH_RANGE   16u  /* patchi/patchf outside 1..np */
#define CLMGB_COL_ADJ_UNSUPPORTED 32u /* step adjoint: the column holds state the adjoint treats as
                                        constant (frac_h2osfc > 0, excess ice, snow without layers) */
#define CLMGB_COL_TAPE_FULL     64u  /* step adjoint: the column's tape (or its substep checkpoints)
                                        overflowed; its adjoints are not computed (raise the entries
                                        of clmgb_reserve_adjoint) */
#define CLMGB_COL_ADJ_REPLAY   128u  /* step adjoint: a replayed substep was not accepted again
                                        (its adjoint is not valid) */
#define CLMGB_COL_QUEUE_WAIT   512u  /* Richards work queue (device status only): a bounded wait for a
                                        deferred column's index ran out and the slot was given back;
                                        the lane that deferred the column finished it itself, so
                                        every result is complete (a record of the slow path) */
#define CLMGB_COL_COPY_WAIT   1024u  /* Richards pre-pass (device status only): a bounded wait for the
                                        tensor copy of a tile of the column records ran out; that
                                        tile's records were not written and the call's results are
                                        not valid */
#define CLMGB_COL_FILTER       256u  /* root sink: the column is in two of the reference's filters
                                        (a pervious road on a natural-vegetation landunit) */

/* ---- compile-time limits of this build ---- */
#define CLMGB_MAX_NLEVSNO   12
#define CLMGB_MAX_NLEVGRND  25
#define CLMGB_MAX_NLEVSOI   25

/* Level counts: mirrors varpar (src/constants/varpar.jl:113-150). */
typedef struct clmgb_varpar {
  int32_t nlevsno;        /* 12 in CLM5 */
  int32_t nlevgrnd;       /* 25 for 20SL_8.5m */
  int32_t nlevsoi;        /* 20 for 20SL_8.5m */
  int32_t nlevurb;        /* urban levels, <= nlevgrnd */
  int32_t nlevmaxurbgrnd; /* max(nlevurb, nlevgrnd); must equal nlevgrnd here */
  int32_t reserved;
} clmgb_varpar;

/* Column / patch / landunit counts and leading dimensions. */
typedef struct clmgb_bounds {
  int64_t nc;   /* columns (length of bounds_col) */
  int64_t np;   /* patches */
  int64_t nl;   /* landunits */
  int64_t ldc;  /* leading dimension of [nc, *] matrices, >= nc */
  int64_t ldp;  /* leading dimension of [np, *] matrices, >= np */
} clmgb_bounds;

/* Snow thermal conductivity method: varctl.snow_thermal_cond_method (varctl.jl:158). */
#define CLMGB_SNOW_JORDAN1991 1
#define CLMGB_SNOW_STURM1997  2

/*
 * Every field soil_temperature! reads or writes for soil/crop/wetland/glacier
 * columns (soil_temperature.jl:358-593).  Field names follow the reference
 * (ColumnData, LandunitData, PatchData, TemperatureData, EnergyFluxData,
 * SoilStateData, WaterStateBulkData, WaterDiagnosticBulkData, WaterFluxBulkData,
 * SolarAbsorbedData, CanopyStateData).  Dimensions: L = nlevsno+nlevmaxurbgrnd,
 * LZ = L+1, G = nlevgrnd, S = nlevsno, S1 = nlevsno+1.
 */
typedef struct clmgb_soiltemp_fields {
  int64_t struct_size;               /* sizeof(clmgb_soiltemp_fields) */
  /* masks and subgrid topology */
  const uint8_t* mask_nolakec;       /* [nc]  filt.nolakec */
  const uint8_t* mask_nolakep;       /* [np]  filt.nolakep */
  const int64_t* col_snl;            /* [nc]  col.snl (0..-nlevsno) */
  const int64_t* col_nbedrock;       /* [nc]  col.nbedrock */
  const int64_t* col_itype;          /* [nc]  col.itype */
  const int64_t* col_landunit;       /* [nc]  col.landunit (1-based) */
  const int64_t* col_patchi;         /* [nc]  col.patchi (1-based, first patch) */
  const int64_t* col_patchf;         /* [nc]  col.patchf (1-based, last patch) */
  const int64_t* lun_itype;          /* [nl]  lun.itype */
  const uint8_t* lun_urbpoi;         /* [nl]  lun.urbpoi */
  const int64_t* patch_column;       /* [np]  patch.column (1-based) */
  const int64_t* patch_landunit;     /* [np]  patch.landunit (1-based) */
  const double*  patch_wtcol;        /* [np]  patch.wtcol */
  const int64_t* frac_veg_nosno;     /* [np]  canopystate.frac_veg_nosno_patch */
  /* geometry */
  const double* dz;                  /* [ldc, L]  col.dz */
  const double* z;                   /* [ldc, L]  col.z */
  const double* zi;                  /* [ldc, LZ] col.zi */
  /* temperature */
  double*  t_soisno;                 /* [ldc, L]  RW */
  double*  t_h2osfc;                 /* [nc]      RW */
  double*  t_grnd;                   /* [nc]      W (read by the lw emission) */
  double*  xmf;                      /* [nc]      W */
  double*  xmf_h2osfc;               /* [nc]      W */
  double*  fact;                     /* [ldc, L]  W */
  double*  c_h2osfc;                 /* [nc]      W */
  int64_t* imelt;                    /* [ldc, L]  W */
  const double* emg;                 /* [nc]  temperature.emg_col */
  /* energy flux */
  const double* htvp;                /* [nc] */
  const double* eflx_bot;            /* [nc] */
  double* eflx_fgr12;                /* [nc]      W */
  double* eflx_fgr;                  /* [ldc, G]  W */
  double* eflx_snomelt;              /* [nc]      W */
  double* eflx_snomelt_r;            /* [nc]      W */
  double* eflx_snomelt_u;            /* [nc]      W (urban only; untouched here) */
  double* eflx_h2osfc_to_snow;       /* [nc]      W */
  double* eflx_gnet;                 /* [np]      W */
  double* dgnetdT;                   /* [np]      W */
  const double* dlrad;               /* [np] */
  const double* cgrnd;               /* [np] */
  const double* eflx_sh_grnd;        /* [np] */
  const double* eflx_sh_snow;        /* [np] */
  const double* eflx_sh_soil;        /* [np] */
  const double* eflx_sh_h2osfc;      /* [np] */
  /* soil state */
  const double* watsat;              /* [ldc, G] */
  const double* bsw;                 /* [ldc, G] */
  const double* sucsat;              /* [ldc, G] */
  const double* tkmg;                /* [ldc, G] */
  const double* tkdry;               /* [ldc, G] */
  const double* csol;                /* [ldc, G] */
  double* thk;                       /* [ldc, L]  W */
  /* water state (bulk) */
  double* h2osoi_liq;                /* [ldc, L]  RW */
  double* h2osoi_ice;                /* [ldc, L]  RW */
  double* excess_ice;                /* [ldc, L]  RW; indexed [c, j] for soil j as the reference does */
  double* h2osno_no_layers;          /* [nc]      RW */
  double* h2osfc;                    /* [nc]      RW */
  double* int_snow;                  /* [nc]      RW */
  /* water diagnostic (bulk) */
  const double* frac_sno_eff;        /* [nc] */
  const double* frac_h2osfc;         /* [nc] */
  double* snow_depth;                /* [nc]      RW */
  double* bw;                        /* [ldc, S]  W */
  double* exice_subs;                /* [ldc, G]  W */
  double* snomelt_accum;             /* [nc]      RW */
  /* water flux (bulk) */
  const double* qflx_evap_soi;       /* [np] */
  const double* qflx_ev_snow;        /* [np] */
  const double* qflx_ev_soil;        /* [np] */
  const double* qflx_ev_h2osfc;      /* [np] */
  double* qflx_snomelt;              /* [nc]      W */
  double* qflx_snofrz;               /* [nc]      W */
  double* qflx_snow_drain;           /* [nc]      W */
  double* qflx_h2osfc_to_ice;        /* [nc]      W */
  double* qflx_snomelt_lyr;          /* [ldc, S]  W */
  double* qflx_snofrz_lyr;           /* [ldc, S]  W */
  /* solar absorbed */
  const double* sabg;                /* [np] */
  const double* sabg_soil;           /* [np] */
  const double* sabg_snow;           /* [np] */
  const double* sabg_lyr;            /* [ldp, S1] */
  double* sabg_chk;                  /* [np]      W */
  /* forcing */
  const double* forc_lwrad;          /* [nc]  atm2lnd forc_lwrad_downscaled_col */
} clmgb_soiltemp_fields;

/* Lower boundary conditions (soil_water_movement.jl:30-34). */
#define CLMGB_BC_HEAD        0
#define CLMGB_BC_FLUX        1
#define CLMGB_BC_ZERO_FLUX   2
#define CLMGB_BC_WATERTABLE  3
#define CLMGB_BC_AQUIFER     4
/* Methods (soil_water_movement.jl:24-27). */
#define CLMGB_ZENGDECKER_2009 0
#define CLMGB_MOISTURE_FORM   1

/* SoilWaterMovementConfig (soil_water_movement.jl:654-671), same defaults. */
typedef struct clmgb_swm_config {
  int32_t soilwater_movement_method;   /* CLMGB_MOISTURE_FORM for this path */
  int32_t upper_boundary_condition;    /* CLMGB_BC_FLUX */
  int32_t lower_boundary_condition;    /* ZERO_FLUX (CLM5 default), FLUX or WATERTABLE */
  int32_t flux_calculation;            /* 1 = inexpensive (default), 42 = expensive */
  double  dtmin;                       /* 60 s */
  double  verySmall;                   /* 1e-8 */
  double  xTolerUpper;                 /* 0.1 */
  double  xTolerLower;                 /* 0.01 */
  double  e_ice;                       /* 6.0 */
} clmgb_swm_config;

/* Every field soil_water! (moisture form) and set_soil_water_fractions! touch. */
typedef struct clmgb_soilwater_fields {
  int64_t struct_size;               /* sizeof(clmgb_soilwater_fields) */
  const uint8_t* mask_hydrology;     /* [nc]  filt.hydrologyc */
  const int64_t* col_nbedrock;       /* [nc] */
  const double* dz;                  /* [ldc, L] */
  const double* z;                   /* [ldc, L] */
  const double* zi;                  /* [ldc, LZ] */
  double* h2osoi_liq;                /* [ldc, L]  RW (soil part) */
  const double* h2osoi_ice;          /* [ldc, L] */
  const double* excess_ice;          /* [ldc, L]  indexed [c, j] for soil j as the reference does */
  const double* watsat;              /* [ldc, G] */
  const double* hksat;               /* [ldc, G] */
  const double* bsw;                 /* [ldc, G] */
  const double* sucsat;              /* [ldc, G] */
  double* eff_porosity;              /* [ldc, G]  W (fractions) */
  double* icefrac;                   /* [ldc, G]  W (fractions), R (moisture form) */
  double* smp_l;                     /* [ldc, G]  W */
  double* hk_l;                      /* [ldc, G]  W */
  const double* qflx_rootsoi;        /* [ldc, nlevsoi] */
  const double* qflx_infl;           /* [nc] */
  const double* zwt;                 /* [nc] */
  double* qcharge;                   /* [nc]  W */
  double* num_substeps;              /* [nc]  W (Float64 as in the reference) */
  const double* smpmin;              /* [nc]  soilstate.smpmin_col, read by compute_qcharge! */
} clmgb_soilwater_fields;

/* compute_effec_rootfrac_and_vert_tran_sink! (soil_water_plant_sink.jl:341-451): the
 * column root fraction and the transpiration sink qflx_rootsoi that soil_water! reads.
 * Patch-level level arrays are [ldp, levels] (element (p, j) at p + (j-1)*ldp). */
typedef struct clmgb_rootsink_fields {
  int64_t struct_size;               /* sizeof(clmgb_rootsink_fields) */
  const uint8_t* mask_hydrology;     /* [nc]  filt.hydrologyc */
  const int64_t* col_itype;          /* [nc] */
  const int64_t* col_landunit;       /* [nc]  1-based */
  const int64_t* lun_itype;          /* [nl] */
  const int64_t* col_patchi;         /* [nc]  1-based first patch */
  const int64_t* col_npatches;       /* [nc] */
  const uint8_t* patch_active;       /* [np] */
  const double* patch_wtcol;         /* [np] */
  const double* rootr_patch;         /* [ldp, G]  levels 1..nlevsoi read */
  const double* qflx_tran_veg_patch; /* [np] */
  const double* qflx_tran_veg_col;   /* [nc] */
  double* rootr_col;                 /* [ldc, G]  W, levels 1..nlevsoi (default method) */
  double* qflx_rootsoi_col;          /* [ldc, nlevsoi]  W */
  /* the hydraulic-stress method only (use_hydrstress != 0; may be NULL otherwise): */
  const double* k_soil_root_patch;   /* [ldp, nlevsoi] */
  const double* smp_l;               /* [ldc, G] */
  const double* vegwp_patch;         /* [ldp, 4]  segment 4 = root */
  const int64_t* frac_veg_nosno;     /* [np] */
  const double* z;                   /* [ldc, L] */
  double* qflx_phs_neg_col;          /* [nc]  W */
  double* qflx_hydr_redist_patch;    /* [np]  W */
} clmgb_rootsink_fields;

/* soilwater_zengdecker2009! (soil_water_movement.jl:1616-1764): the fields of the
 * Zeng & Decker (2009) method, which soil_water! selects with use_aquifer_layer. */
typedef struct clmgb_zd09_fields {
  int64_t struct_size;               /* sizeof(clmgb_zd09_fields) */
  const uint8_t* mask_hydrology;     /* [nc] */
  const double* dz;                  /* [ldc, L] */
  const double* z;                   /* [ldc, L] */
  const double* zi;                  /* [ldc, LZ] */
  const double* t_soisno;            /* [ldc, L] */
  double* h2osoi_liq;                /* [ldc, L]  RW (soil part) */
  const double* h2osoi_ice;          /* [ldc, L] */
  const double* h2osoi_vol;          /* [ldc, G] */
  const double* watsat;              /* [ldc, G] */
  const double* hksat;               /* [ldc, G] */
  const double* bsw;                 /* [ldc, G] */
  const double* sucsat;              /* [ldc, G] */
  const double* smpmin;              /* [nc] */
  double* icefrac;                   /* [ldc, G]  W */
  double* smp_l;                     /* [ldc, G]  W */
  double* hk_l;                      /* [ldc, G]  W */
  const double* qflx_rootsoi;        /* [ldc, nlevsoi] */
  const double* qflx_infl;           /* [nc] */
  const double* zwt;                 /* [nc] */
  double* qcharge;                   /* [nc]  W */
  double* qflx_deficit;              /* [nc]  W */
} clmgb_zd09_fields;

/* The use_flexibleCN branch of soil_water! (soil_water_movement.jl:1812-1843): after the
 * solve, negative liquid water of soil levels 1..nlevsoi-1 is raised to watmin = 0.001 mm
 * from the level below, that of level nlevsoi from the aquifer store wa, and h2osoi_vol
 * is formed from liquid water and ice on levels 1..nlevsoi. */
typedef struct clmgb_flexcn_fields {
  int64_t struct_size;               /* sizeof(clmgb_flexcn_fields) */
  const uint8_t* mask_hydrology;     /* [nc] */
  const double* dz;                  /* [ldc, L] */
  double* h2osoi_liq;                /* [ldc, L]  RW (soil part) */
  const double* h2osoi_ice;          /* [ldc, L] */
  double* h2osoi_vol;                /* [ldc, G]  W (levels 1..nlevsoi) */
  double* wa;                        /* [nc]  RW: waterstatebulk.ws.wa_col */
} clmgb_flexcn_fields;

/* soil_fluxes! (soil_fluxes.jl:553-697): the surface fluxes corrected to the new ground
 * temperature, the evaporation partition, totals, outgoing longwave and the soil
 * energy balance error.  [np] patch vectors, [nc] column vectors, [nl] landunits. */
typedef struct clmgb_soilflux_fields {
  int64_t struct_size;               /* sizeof(clmgb_soilflux_fields) */
  const uint8_t* mask_nolakec;       /* [nc] */
  const uint8_t* mask_nolakep;       /* [np] */
  const uint8_t* mask_urbanp;        /* [np] */
  const int64_t* col_snl;            /* [nc] */
  const int64_t* col_itype;          /* [nc] */
  const int64_t* col_patchi;         /* [nc]  1-based */
  const int64_t* col_patchf;         /* [nc]  1-based */
  const int64_t* lun_itype;          /* [nl] */
  const uint8_t* lun_urbpoi;         /* [nl] */
  const int64_t* patch_column;       /* [np]  1-based */
  const int64_t* patch_landunit;     /* [np]  1-based */
  const double* patch_wtcol;         /* [np] */
  const int64_t* frac_veg_nosno;     /* [np] */
  const double* frac_sno_eff;        /* [nc] */
  const double* frac_h2osfc;         /* [nc] */
  const double* t_ssbef;             /* [ldc, L] */
  const double* t_h2osfc_bef;        /* [nc] */
  const double* t_grnd;              /* [nc] */
  const double* t_h2osfc;            /* [nc] */
  const double* emg;                 /* [nc] */
  const double* t_soisno;            /* [ldc, L] */
  const double* fact;                /* [ldc, L] */
  const double* h2osoi_liq;          /* [ldc, L] */
  const double* h2osoi_ice;          /* [ldc, L] */
  const double* htvp;                /* [nc] */
  const double* xmf;                 /* [nc] */
  const double* xmf_h2osfc;          /* [nc] */
  const double* c_h2osfc;            /* [nc] */
  const double* eflx_h2osfc_to_snow; /* [nc] */
  const double* eflx_building_heat_errsoi; /* [nc] */
  const double* forc_lwrad;          /* [nc] */
  double* errsoi_col;                /* [nc]  W */
  const double* cgrnds;              /* [np] */
  const double* cgrndl;              /* [np] */
  const double* sabg;                /* [np] */
  const double* sabg_soil;           /* [np] */
  const double* sabg_snow;           /* [np] */
  const double* dlrad;               /* [np] */
  const double* ulrad;               /* [np] */
  const double* eflx_sh_veg;         /* [np] */
  const double* eflx_sh_stem;        /* [np] */
  const double* eflx_wasteheat;      /* [np] */
  const double* eflx_heat_from_ac;   /* [np] */
  const double* eflx_traffic;        /* [np] */
  const double* eflx_ventilation;    /* [np] */
  const double* qflx_evap_veg;       /* [np] */
  const double* qflx_tran_veg;       /* [np] */
  double* eflx_sh_grnd;              /* [np]  RW */
  double* qflx_evap_soi;             /* [np]  RW */
  double* qflx_ev_soil;              /* [np]  RW */
  double* qflx_ev_h2osfc;            /* [np]  RW */
  double* qflx_ev_snow;              /* [np]  RW */
  double* eflx_lwrad_net;            /* [np]  RW (read by urban patches) */
  double* eflx_lwrad_out;            /* [np]  RW */
  double* eflx_lwrad_net_u;          /* [np]  RW */
  double* eflx_sh_tot;               /* [np]  W */
  double* eflx_sh_tot_r;             /* [np]  W */
  double* eflx_sh_tot_u;             /* [np]  W */
  double* eflx_lh_tot;               /* [np]  W */
  double* eflx_lh_tot_r;             /* [np]  W */
  double* eflx_lh_tot_u;             /* [np]  W */
  double* eflx_lh_vege;              /* [np]  W */
  double* eflx_lh_vegt;              /* [np]  W */
  double* eflx_lh_grnd;              /* [np]  W */
  double* eflx_soil_grnd;            /* [np]  W */
  double* eflx_soil_grnd_r;          /* [np]  W */
  double* eflx_soil_grnd_u;          /* [np]  W */
  double* eflx_lwrad_net_r;          /* [np]  W */
  double* eflx_lwrad_out_r;          /* [np]  W */
  double* eflx_lwrad_out_u;          /* [np]  W */
  double* errsoi_patch;              /* [np]  W */
  double* t_skin;                    /* [np]  W */
  double* qflx_evap_tot;             /* [np]  W */
  double* qflx_evap_can;             /* [np]  W */
  double* qflx_liqevap_from_top_layer;   /* [np]  W */
  double* qflx_solidevap_from_top_layer; /* [np]  W */
  double* qflx_soliddew_to_top_layer;    /* [np]  W */
  double* qflx_liqdew_to_top_layer;      /* [np]  W */
} clmgb_soilflux_fields;

/* ---- surface hydrology before the soil solve (clm_driver.jl:1938-2007) ----
 * The steps of the driver between set_soil_water_fractions! and the root sink, each a
 * per-column update, run by clmgb_surface_hydrology in the driver's order for the
 * stages selected by a mask of these bits:                                          */
#define CLMGB_SH_FLOODC          1u   /* set_floodc! (soil_hydrology.jl:430-442; kernel :139-152) */
#define CLMGB_SH_SAT_EXCESS      2u   /* saturated_excess_runoff! (sat_excess_runoff.jl:329-365; kernel :246-300) */
#define CLMGB_SH_QFLX_INPUTS     4u   /* set_qflx_inputs! (soil_hydrology.jl:456-485; kernel :160-187) */
#define CLMGB_SH_INFL_EXCESS     8u   /* infiltration_excess_runoff! (infilt_excess_runoff.jl:142-211, :241-274) */
#define CLMGB_SH_ROUTE          16u   /* route_infiltration_excess! (soil_hydrology.jl:500-525; kernel :199-225) */
#define CLMGB_SH_UPDATE_H2OSFC  32u   /* update_h2osfc! (surface_water.jl:462-520; kernels :279-450) */
#define CLMGB_SH_INFILTRATION   64u   /* infiltration! (soil_hydrology.jl:538-552; kernel :236-243) */
#define CLMGB_SH_TOTAL_RUNOFF  128u   /* total_surface_runoff! (soil_hydrology.jl:567-604; kernels :250-301) */
#define CLMGB_SH_URBAN_PONDING 256u   /* update_urban_ponding! (soil_hydrology.jl:618-640; kernel :316-338) */
#define CLMGB_SH_ALL           511u

/* saturated_excess_runoff! fsat methods (sat_excess_runoff.jl:31-32) and
 * infiltration_excess_runoff! qinmax methods (infilt_excess_runoff.jl:40-41). */
#define CLMGB_FSAT_TOPMODEL 1
#define CLMGB_FSAT_VIC      2
#define CLMGB_QINMAX_NONE   0
#define CLMGB_QINMAX_HKSAT  1

/* The scalars of those routines: parameters, method flags and keyword arguments. */
typedef struct clmgb_surfhyd_config {
  int64_t struct_size;                /* sizeof(clmgb_surfhyd_config) */
  int64_t ng;                         /* gridcells: length of qflx_floodg */
  int32_t fsat_method;                /* SaturatedExcessRunoffData.fsat_method */
  int32_t crop_fsat_equals_zero;      /* keyword of saturated_excess_runoff! (default 0) */
  int32_t hillslope_fsat_equals_zero; /* keyword of saturated_excess_runoff! (default 0) */
  int32_t qinmax_method;              /* InfiltrationExcessRunoffData.qinmax_method */
  int32_t h2osfcflag;                 /* SoilHydrologyData.h2osfcflag, read by route_infiltration_excess! */
  int32_t update_h2osfcflag;          /* the h2osfcflag keyword of update_h2osfc! (the driver leaves it 1) */
  double  fff;                        /* sat_excess_runoff_params.fff, TOPModel decay factor (1/m) */
  double  e_ice;                      /* infilt_excess_params.e_ice (6.0) */
  double  pc;                         /* SURFACE_WATER_PC (0.4) */
  double  mu;                         /* SURFACE_WATER_MU (0.13889) */
  double  pondmx_urban;               /* PONDMX_URBAN (1.0 mm) */
} clmgb_surfhyd_config;

/* Every field those routines read or write.  [nc] column vectors, [nl] landunits,
 * [ng] gridcells; icefrac/hksat [ldc, G] soil levels; h2osoi_liq [ldc, L] (the top
 * soil level is row nlevsno). */
typedef struct clmgb_surfhyd_fields {
  int64_t struct_size;                /* sizeof(clmgb_surfhyd_fields) */
  const uint8_t* mask_nolakec;        /* [nc]  filt.nolakec (set_floodc!) */
  const uint8_t* mask_hydrology;      /* [nc]  filt.hydrologyc */
  const uint8_t* mask_urban;          /* [nc]  filt.urbanc (total_surface_runoff!, update_urban_ponding!) */
  const int64_t* col_snl;             /* [nc] */
  const int64_t* col_itype;           /* [nc] */
  const int64_t* col_landunit;        /* [nc]  1-based */
  const int64_t* col_gridcell;        /* [nc]  1-based */
  const uint8_t* col_urbpoi;          /* [nc] */
  const uint8_t* col_is_hillslope;    /* [nc] */
  const uint8_t* col_active;          /* [nc] */
  const int64_t* col_cold;            /* [nc]  ISPVAL (-9999) when none */
  const int64_t* lun_itype;           /* [nl] */
  const double* qflx_floodg;          /* [ng] */
  const double* frost_table;          /* [nc] */
  const double* zwt;                  /* [nc] */
  const double* zwt_perched;          /* [nc] */
  const double* wtfact;               /* [nc] */
  const double* b_infil;              /* [nc]  VIC */
  const double* top_max_moist;        /* [nc]  VIC */
  const double* top_moist_limited;    /* [nc]  VIC */
  const double* icefrac;              /* [ldc, G] */
  const double* hksat;                /* [ldc, G] */
  const double* frac_sno_eff;         /* [nc] */
  const double* frac_h2osfc;          /* [nc] */
  const double* frac_h2osfc_nosnow;   /* [nc] */
  const double* h2osfc_thresh;        /* [nc] */
  const double* topo_slope;           /* [nc]  degrees */
  const double* qflx_rain_plus_snomelt; /* [nc] */
  const double* qflx_snow_h2osfc;     /* [nc] */
  const double* qflx_liqevap_from_top_layer; /* [nc] */
  const double* qflx_ev_soil;         /* [nc] */
  const double* qflx_ev_h2osfc;       /* [nc] */
  double* qflx_floodc;                /* [nc]  W (set_floodc!), R after */
  double* fsat;                       /* [nc]  W */
  double* fcov;                       /* [nc]  W */
  double* qflx_sat_excess_surf;       /* [nc]  W */
  double* qflx_top_soil;              /* [nc]  W */
  double* qflx_in_soil;               /* [nc]  W */
  double* qflx_top_soil_to_h2osfc;    /* [nc]  W */
  double* qinmax;                     /* [nc]  W */
  double* qflx_infl_excess;           /* [nc]  W */
  double* qflx_in_soil_limited;       /* [nc]  W */
  double* qflx_in_h2osfc;             /* [nc]  W */
  double* qflx_infl_excess_surf;      /* [nc]  W */
  double* h2osfc;                     /* [nc]  RW */
  double* qflx_h2osfc_surf;           /* [nc]  W */
  double* qflx_h2osfc_drain;          /* [nc]  W */
  double* qflx_infl;                  /* [nc]  W */
  double* qflx_surf;                  /* [nc]  W */
  double* xs_urban;                   /* [nc]  RW */
  double* h2osoi_liq;                 /* [ldc, L]  RW (top soil level of urban columns) */
} clmgb_surfhyd_fields;

/* ---- snow layer dynamics (clm_driver.jl:2146-2200) ----
 * The snow-layer steps of clm_drv_core! after the soil solve, per column over the snow
 * filter, selected by a mask of these bits and run in this order:                  */
#define CLMGB_SL_COMPACTION  1u   /* snow_compaction! (snow_hydrology.jl:1203-1398, 1412-1500) */
#define CLMGB_SL_COMBINE     2u   /* combine_snow_layers! (:1584-1926) with combo_scalar (:1960-2000) */
#define CLMGB_SL_DIVIDE      4u   /* divide_snow_layers! (:2057-2286), mass_weighted_snow_radius (:2021-2031) */
#define CLMGB_SL_ZERO_EMPTY  8u   /* zero_empty_snow_layers! (:2298-2329) */
#define CLMGB_SL_FILTER     16u   /* build_snow_filter! (:2488-2510): snow/no-snow filters from snl */
#define CLMGB_SL_ALL        31u

#define CLMGB_OVERBURDEN_ANDERSON1976 1   /* snow_hydrology.jl:78-79 */
#define CLMGB_OVERBURDEN_VIONNET2012  2

/* The parameters and switches of those routines (SnowHydrologyParams, snow_hydrology.jl:43-63;
 * the module switches :90-101; varctl.use_subgrid_fluxes). */
typedef struct clmgb_snowlayer_config {
  int64_t struct_size;                /* sizeof(clmgb_snowlayer_config) */
  int64_t ng;                         /* gridcells: length of forc_wind */
  int32_t use_subgrid_fluxes;         /* varctl.use_subgrid_fluxes (1) */
  int32_t overburden_method;          /* OVERBURDEN_COMPACTION_METHOD (Anderson 1976) */
  int32_t wind_dependent_snow_density;/* WIND_DEPENDENT_SNOW_DENSITY (0) */
  int32_t is_lake;                    /* divide_snow_layers!'s is_lake (0 in clm_drv_core!) */
  double  int_snow_max;               /* SCF int_snow_max (2000 mm) */
  double  overburden_compress_tfactor;/* 0.08 1/K */
  double  upplim_destruct_metamorph;  /* 100 kg/m3 */
  double  eta0_anderson;              /* 9.0e5 kg s/m2 */
  double  eta0_vionnet;               /* 7.62237e6 kg s/m2 */
  double  ceta;                       /* 250 kg/m3 */
  double  drift_gs;                   /* 0.35 */
  double  rho_min;                    /* 50 kg/m3 */
  double  rho_max;                    /* 350 kg/m3 */
  double  tau_ref;                    /* 172800 s */
  double  snw_rds_min;                /* 54.526 microns */
  double  snw_rds_max;                /* SNW_RDS_MAX, 1500 microns */
  double  dzmin_1;                    /* SNOW_DZMIN_1 (0.010 m) */
  double  dzmin_2;                    /* SNOW_DZMIN_2 (0.015 m) */
  double  dzmax_l_1;                  /* SNOW_DZMAX_L_1 (0.03 m) */
  double  dzmax_l_2;                  /* SNOW_DZMAX_L_2 (0.07 m) */
  double  dzmax_u_1;                  /* SNOW_DZMAX_U_1 (0.02 m) */
  double  dzmax_u_2;                  /* SNOW_DZMAX_U_2 (0.05 m); deeper levels follow init_snow_layers! (:2357-2377) */
} clmgb_snowlayer_config;

/* Every field those routines read or write.  [ldc, S] arrays hold the nlevsno snow
 * levels (CLM.jl's [nc, nlevsno] snow matrices, or the snow part of a longer one);
 * [ldc, L] and [ldc, LZ] are the combined snow+soil arrays. */
typedef struct clmgb_snowlayer_fields {
  int64_t struct_size;                /* sizeof(clmgb_snowlayer_fields) */
  uint8_t* mask_snow;                 /* [nc]  RW: filt.snowc (rebuilt by CLMGB_SL_FILTER) */
  uint8_t* mask_nosnow;               /* [nc]  W: filt.nosnowc */
  const uint8_t* mask_nolakec;        /* [nc]  filt.nolakec (CLMGB_SL_FILTER) */
  int64_t* col_snl;                   /* [nc]  RW */
  const int64_t* col_landunit;        /* [nc]  1-based */
  const int64_t* col_gridcell;        /* [nc]  1-based */
  const int64_t* lun_itype;           /* [nl] */
  const uint8_t* lun_lakpoi;          /* [nl] */
  const uint8_t* lun_urbpoi;          /* [nl] */
  const double* forc_wind;            /* [ng] */
  const double* n_melt;               /* [nc]  SCF melt shape parameter */
  const double* frac_h2osfc;          /* [nc] */
  double* frac_sno;                   /* [nc]  RW */
  double* frac_sno_eff;               /* [nc]  RW */
  double* int_snow;                   /* [nc]  RW */
  double* h2osno_no_layers;           /* [nc]  W */
  double* snow_depth;                 /* [nc]  W */
  double* qflx_sl_top_soil;           /* [nc]  W */
  double* dz;                         /* [ldc, L]  RW */
  double* z;                          /* [ldc, L]  RW */
  double* zi;                         /* [ldc, LZ] RW */
  double* t_soisno;                   /* [ldc, L]  RW */
  double* h2osoi_ice;                 /* [ldc, L]  RW (snow levels and soil level 1) */
  double* h2osoi_liq;                 /* [ldc, L]  RW (snow levels and soil level 1) */
  const int64_t* imelt;               /* [ldc, S] */
  const double* swe_old;              /* [ldc, S] */
  const double* frac_iceold;          /* [ldc, S] */
  double* snw_rds;                    /* [ldc, S]  RW */
  double* mss_bcphi;                  /* [ldc, S]  RW */
  double* mss_bcpho;                  /* [ldc, S]  RW */
  double* mss_ocphi;                  /* [ldc, S]  RW */
  double* mss_ocpho;                  /* [ldc, S]  RW */
  double* mss_dst1;                   /* [ldc, S]  RW */
  double* mss_dst2;                   /* [ldc, S]  RW */
  double* mss_dst3;                   /* [ldc, S]  RW */
  double* mss_dst4;                   /* [ldc, S]  RW */
} clmgb_snowlayer_fields;

/* ---- lake temperature (lake_temperature.jl:1016-1295) ---- */
/* The lake configuration: varpar.nlevlak and the lake_con sub-options. */
typedef struct clmgb_lake_config {
  int64_t struct_size;                /* sizeof(clmgb_lake_config) */
  int32_t nlevlak;                    /* varpar.nlevlak (10), at most CLMGB_MAX_NLEVLAK */
  int32_t use_lch4;                   /* varctl.use_lch4: lake resistance and CH4 conductance */
  int32_t lakepuddling;               /* lake_con.lakepuddling (0) */
  int32_t lake_no_ed;                 /* lake_con.lake_no_ed (0) */
  double  deepmixing_depthcrit;       /* lake_con.deepmixing_depthcrit (25 m) */
  double  deepmixing_mixfact;         /* lake_con.deepmixing_mixfact (10) */
  double  lake_puddle_thick;          /* lake_con.lake_puddle_thick (0.2 m) */
} clmgb_lake_config;
#define CLMGB_MAX_NLEVLAK 16

/* Every field lake_temperature! reads or writes.  K = nlevlak lake levels; each lake
 * column has one patch, col_patchi (CLM's col.patchi). */
typedef struct clmgb_lake_fields {
  int64_t struct_size;                /* sizeof(clmgb_lake_fields) */
  const uint8_t* mask_lakec;          /* [nc]  filt.lakec */
  const uint8_t* mask_lakep;          /* [np]  filt.lakep */
  const int64_t* col_patchi;          /* [nc]  1-based */
  const int64_t* patch_column;        /* [np]  1-based */
  const int64_t* col_snl;             /* [nc] */
  const double* dz;                   /* [ldc, L] */
  const double* z;                    /* [ldc, L] */
  const double* zi;                   /* [ldc, LZ] */
  const double* dz_lake;              /* [ldc, K] */
  const double* z_lake;               /* [ldc, K] */
  const double* lakedepth;            /* [nc] */
  const double* watsat;               /* [ldc, G] */
  const double* tksatu;               /* [ldc, G] */
  const double* tkmg;                 /* [ldc, G] */
  const double* tkdry;                /* [ldc, G] */
  const double* csol;                 /* [ldc, G] */
  const double* t_grnd;               /* [nc] */
  const double* etal;                 /* [nc] */
  const double* ks;                   /* [nc] */
  const double* ws;                   /* [nc] */
  const double* lake_raw;             /* [nc] */
  double* t_soisno;                   /* [ldc, L]  RW */
  double* t_lake;                     /* [ldc, K]  RW */
  double* h2osoi_liq;                 /* [ldc, L]  RW */
  double* h2osoi_ice;                 /* [ldc, L]  RW */
  double* h2osno_no_layers;           /* [nc]  RW */
  double* snow_depth;                 /* [nc]  RW */
  double* frac_iceold;                /* [ldc, S]  W */
  double* betaprime;                  /* [nc]  W */
  double* lake_icefrac;               /* [ldc, K]  RW */
  double* lake_icefracsurf;           /* [nc]  W */
  double* lake_icethick;              /* [nc]  W */
  double* savedtke1;                  /* [nc]  W */
  double* lakeresist;                 /* [nc]  W (use_lch4) */
  double* grnd_ch4_cond;              /* [nc]  W (use_lch4) */
  double* qflx_snomelt;               /* [nc]  W */
  double* qflx_snofrz;                /* [nc]  W */
  double* qflx_snow_drain;            /* [nc]  W */
  double* qflx_snomelt_lyr;           /* [ldc, S]  W */
  double* qflx_snofrz_lyr;            /* [ldc, S]  W */
  int64_t* imelt;                     /* [ldc, S]  W */
  double* eflx_snomelt;               /* [nc]  W */
  double* errsoi_col;                 /* [nc]  W */
  const double* sabg;                 /* [np] */
  const double* sabg_lyr;             /* [ldp, S1] */
  const double* fsds_nir_d;           /* [np] */
  const double* fsds_nir_i;           /* [np] */
  const double* fsr_nir_d;            /* [np] */
  const double* fsr_nir_i;            /* [np] */
  double* eflx_gnet;                  /* [np]  RW */
  double* eflx_sh_tot;                /* [np]  RW */
  double* eflx_sh_grnd;               /* [np]  RW */
  double* eflx_soil_grnd;             /* [np]  RW */
} clmgb_lake_fields;

typedef struct clmgb_handle_s* clmgb_handle;

/* ---- library / handle ---- */
int32_t     clmgb_abi_version(void);
const char* clmgb_build_info(void);
const char* clmgb_strerror(int32_t code);
/* Create a handle bound to the current CUDA device; allocates the handle's device
 * status word.  Returns CLMGB_OK and writes *out. */
int32_t clmgb_create(const clmgb_varpar* vp, clmgb_handle* out);
int32_t clmgb_destroy(clmgb_handle h);
/* Copy the OR of all per-column status bits since the last reset to *status (host
 * pointer; synchronises `stream`) and optionally clear it. */
int32_t clmgb_device_status(clmgb_handle h, void* stream, uint32_t* status, int32_t reset);
int32_t clmgb_last_cuda_error(clmgb_handle h);

/* ---- tunables (clmgb_set_option / clmgb_get_option keys) ---- */
#define CLMGB_OPT_STEP_SCHEDULE        1  /* how the Richards solve is scheduled: */
#define   CLMGB_SCHEDULE_FUSED         0  /*   one column per thread, whole step in one kernel */
#define   CLMGB_SCHEDULE_QUEUE         1  /*   persistent kernel fed by a device work queue (default) */
#define   CLMGB_SCHEDULE_WAVES         2  /*   cooperative kernel, all columns in synchronous rounds of
                                              uniform phases (needs clmgb_reserve; otherwise QUEUE runs) */
#define CLMGB_OPT_QUEUE_BLOCKS_PER_SM  2  /* resident blocks per SM of the queue kernel (0 = occupancy limit) */
#define CLMGB_OPT_QUEUE_OCCUPANCY      3  /* read-only: occupancy limit of the queue kernel */
#define CLMGB_OPT_NUM_SMS              4  /* read-only: SMs of the handle's device */
#define CLMGB_OPT_QUEUE_ORDER          5  /* with reserved scratch: 1 = hand out columns longest-expected-first
                                             (by the previous call's num_substeps, default), 0 = index order */
#define CLMGB_OPT_RESERVED_COLUMNS     6  /* read-only: columns covered by clmgb_reserve */
#define CLMGB_OPT_WAVES_BLOCKS_PER_SM  7  /* co-resident blocks per SM of the wave kernel (0 = occupancy limit) */
#define CLMGB_OPT_WAVES_OCCUPANCY      8  /* read-only: occupancy limit of the wave kernel (0 = unavailable) */
#define CLMGB_OPT_ADJ_TAPE_USED        9  /* read-only (synchronises): most tape entries one column used in
                                             clmgb_column_step_vjp since clmgb_reserve_adjoint */
#define CLMGB_OPT_ADJ_TAPE_SLOTS      10  /* read-only: tape slots (concurrent columns) reserved */
#define CLMGB_OPT_ADJ_TAPE_ENTRIES    11  /* read-only: tape entries per slot reserved */
#define CLMGB_OPT_ADJ_RICHARDS        12  /* how clmgb_column_step_vjp reverses the Richards substeps: */
#define   CLMGB_ADJ_RICHARDS_CLOSED_FORM 0 /*   hand-written reverse of each accepted substep (default) */
#define   CLMGB_ADJ_RICHARDS_RECORDED    1 /*   each substep replayed through the recording scalar */
#define CLMGB_OPT_ADJ_SOIL_TEMPERATURE 13 /* how clmgb_column_step_vjp reverses soil_temperature!: */
#define   CLMGB_ADJ_ST_CLOSED_FORM       0 /*   hand-written reverse of every stage, no tape (default;
                                                 used when CLMGB_OPT_ADJ_RICHARDS is closed form too) */
#define   CLMGB_ADJ_ST_RECORDED          1 /*   replayed through the recording scalar and swept */
#define CLMGB_OPT_QUEUE_FRESH_BATCH   14 /* work-queue Richards kernel: lanes whose substep was accepted wait
                                            for the hydraulic block until this many lanes of the warp need it
                                            (or no lane can attempt), then run it together (default 4); 0 = at
                                            once.  Results do not depend on it. */
#define CLMGB_OPT_QUEUE_DEFER         16 /* work-queue Richards kernel with reserved scratch: a column not done
                                            after this many attempts (default 22) leaves the queue at its next
                                            accepted substep and is finished by one warp (one level per lane);
                                            0 = off.  Results do not depend on it. */
#define CLMGB_OPT_QUEUE_PACKED_REFRESH 17 /* work-queue Richards kernel with reserved scratch: 1 (default) = the
                                            warp runs the hydraulic refresh of its waiting lanes' columns
                                            together, column levels spread over the 32 lanes; 0 = each lane
                                            runs its own.  Results do not depend on it. */
#define CLMGB_OPT_ATTEMPT_CAP         18 /* Richards substep attempts after which a column stops with
                                            CLMGB_COL_SUBSTEP_CAP (1..4096, default 4096: never reached by a
                                            valid configuration, whose attempts dtmin bounds) */
#define CLMGB_OPT_QUEUE_POLL_LIMIT    19 /* polls of a deferred column's list slot before the finishing warp
                                            gives the slot back to the deferring lane (0..2^20, default
                                            2^20).  Results do not depend on it. */
#define CLMGB_OPT_QUEUE_PUBLISH_DELAY 20 /* for tests of the bounded wait: a deferring lane counts an even
                                            list slot published before writing the column's index, and
                                            writes it once a finishing warp has taken the slot or after
                                            this many ns; a warp with nothing to finish keeps looking for
                                            as long (0..1e7, default 0: index first, no lingering).  Results
                                            do not depend on it. */
#define CLMGB_OPT_COUNT_WORK          21 /* 1: the work-queue Richards kernel with reserved scratch (packed
                                            refresh) and its warp-per-column finish count, over the calls that
                                            follow, the levels of every substep attempt and of every hydraulic
                                            refresh (setting 1 zeroes the counts; 0 = off, the default) */
#define CLMGB_OPT_WORK_LEVEL_ATTEMPTS 22 /* read-only (synchronises): that count of attempt levels */
#define CLMGB_OPT_WORK_LEVEL_REFRESHES 23 /* read-only (synchronises): that count of refreshed levels */
#define CLMGB_OPT_RECORDS_TMA         24 /* the Richards pre-pass stages each tile of 32 columns with 2-D
                                            tensor copies (TMA, 1, the default) or with plain loads (0);
                                            arrays the tensor copy cannot address (a base address or a
                                            row stride not a multiple of 16 bytes) take plain loads.
                                            Results do not depend on it. */
#define CLMGB_OPT_RECORDS_TMA_USED    25 /* read-only: 1 if the last pre-pass of this handle used tensor
                                            copies, 0 if it took plain loads */
#define CLMGB_OPT_TRIDIAG_METHOD      26 /* solver of clmgb_tridiagonal_multi: CLMGB_TRIDIAG_THOMAS (default)
                                            or CLMGB_TRIDIAG_PCR */
#define CLMGB_OPT_ST_BLOCK            27 /* columns per block of the soil-temperature kernels, sorted together
                                            by snow-layer count so that a warp's lanes run loops of the same
                                            length: 128, 320 (default) or 640.  Results do not depend on it. */
#define CLMGB_TRIDIAG_THOMAS 0
#define CLMGB_TRIDIAG_PCR    1
#define CLMGB_OPT_COLUMN_BASE         15 /* global 0-based index of column 0 of the arrays the next calls
                                            receive (default 0).  A caller that runs a column range [c0, c1)
                                            passes column arrays advanced by c0 (same ldc) and the patch
                                            arrays whole, since col_patchi/col_patchf and patch_column
                                            hold global indices, and sets this to c0. */
int32_t clmgb_set_option(clmgb_handle h, int32_t key, int64_t value);
/* Gives the handle per-column scratch for up to max_nc columns (about 136*nlevsoi + 80
 * bytes per column): the Richards solve then forms the ice impedances in a uniform
 * pre-pass, gathers each column's refresh inputs and water into one contiguous record
 * (the solve keeps the column's water, smp_l and hk_l there and a post-pass writes
 * them to the state), hands out columns longest-expected-first, and the WAVES
 * schedule becomes available.  Calls with more columns
 * than reserved run without it.  Synchronises the device; call it at set-up, not
 * inside stream capture. */
int32_t clmgb_reserve(clmgb_handle h, int64_t max_nc);
int32_t clmgb_get_option(clmgb_handle h, int32_t key, int64_t* value);

/* Evaluates the library's binary64 log (op 0), exp (1), pow (2), log10 (3), sin (4), acos (5)
 * or division x / y (6, the kernels' division: the IEEE quotient, formed on the integer pipes)
 * elementwise on device arrays; y is read for pow and division only.  The oracle and
 * the tests use it to check that the GPU rounds exactly as the CPU build does. */
int32_t clmgb_math_eval(clmgb_handle h, int32_t op, int64_t n, const double* x, const double* y,
                        double* out, void* stream);

/* ---- drop-in entry points ---- */

/* soil_temperature! (soil_temperature.jl:358) for non-urban, non-lake columns.
 * snow_method: CLMGB_SNOW_JORDAN1991 | CLMGB_SNOW_STURM1997;
 * use_excess_ice must be 0 (varctl default, varctl.jl:215);
 * col_status: optional [nc] uint32 per-column status out (may be NULL). */
int32_t clmgb_soil_temperature(clmgb_handle h, const clmgb_bounds* b,
                               const clmgb_soiltemp_fields* f, double dtime,
                               int32_t snow_method, int32_t use_excess_ice,
                               uint32_t* col_status, void* stream);

/* set_soil_water_fractions! (soil_hydrology.jl:394-416; kernel :110-130). */
int32_t clmgb_soil_water_fractions(clmgb_handle h, const clmgb_bounds* b,
                                   const clmgb_soilwater_fields* f, void* stream);

/* soil_water! (soil_water_movement.jl:1780) with the moisture-form method:
 * soilwater_moisture_form! (:1532-1601), i.e. soilwm_moisture_form_solve! (:1498) and,
 * with the BC_WATERTABLE lower boundary (use_aquifer_layer, :707-710), compute_qcharge!
 * (:1153-1215) over the solved state with the zeroed dwat/smp/imped rows the reference
 * passes (:1575-1598): qcharge of every column whose water table lies within the soil
 * column (jwt < nlevsoi) is overwritten.  ZENGDECKER_2009 -> CLMGB_ERR_UNSUPPORTED (use
 * clmgb_soil_water_zd09); BC_AQUIFER -> CLMGB_ERR_CONFIG (soilwm_moisture_form_solve!
 * rejects it with error(), :1502-1505).  Every entry point below that runs the moisture-form solve
 * (column steps, their adjoints, the warm start, the sample recorder, the allocation-free
 * solve) applies the same compute_qcharge! pass. */
int32_t clmgb_soil_water(clmgb_handle h, const clmgb_bounds* b,
                         const clmgb_soilwater_fields* f, const clmgb_swm_config* cfg,
                         double dtime, uint32_t* col_status, void* stream);

/* The use_flexibleCN branch at the end of soil_water! (soil_water_movement.jl:1812-1843),
 * one thread per hydrology column; a caller running soil_water! with use_flexibleCN calls
 * it right after clmgb_soil_water (or clmgb_soil_water_zd09). */
int32_t clmgb_soil_water_flexible_cn(clmgb_handle h, const clmgb_bounds* b, const clmgb_flexcn_fields* f,
                                     void* stream);

/* soil_fluxes! (soil_fluxes.jl:553-697) in its loop order: the ground temperature
 * change tinc (per column), the flux correction, evaporation partition and limit,
 * totals, errsoi and outgoing longwave (per patch), then errsoi_col as the wtcol-weighted
 * patch sum in ascending patch order (the reference's p2c), and urban t_skin. */
int32_t clmgb_soil_fluxes(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilflux_fields* f, double dtime,
                          void* stream);

/* The surface hydrology of clm_drv_core! before the root sink and soil_water!
 * (clm_driver.jl:1938-2007), one thread per column: the CLMGB_SH_* stages in `stages`
 * run in the driver's order, each over its own filter (nolakec for set_floodc!, urbanc
 * for the urban part of total_surface_runoff! and update_urban_ponding!, hydrologyc for
 * the rest), with the results of the reference's calls one by one.  A stage reads what
 * an earlier selected stage wrote from registers and what no selected stage wrote from
 * memory, so any subset is the same sequence of reference calls.  Only the pointers of
 * the selected stages are required.  fsat_method and qinmax_method outside their sets
 * -> CLMGB_ERR_CONFIG, as the reference's error().  Gridcell and landunit indices out of
 * range set CLMGB_COL_PATCH_RANGE in the device status and skip the column. */
int32_t clmgb_surface_hydrology(clmgb_handle h, const clmgb_bounds* b, const clmgb_surfhyd_fields* f,
                                const clmgb_surfhyd_config* cfg, uint32_t stages, double dtime, void* stream);

/* The snow layer dynamics of clm_drv_core! after the soil solve (clm_driver.jl:2146-2200),
 * one thread per snow-filter column: the CLMGB_SL_* stages in `stages` run in order on
 * the column's snow levels held on chip, with the results of the reference's calls one
 * after another (the layer thresholds dzmin/dzmax_l/dzmax_u are built from the config
 * as init_snow_layers! builds them).  Only the pointers of the selected stages are
 * required (the arrays each reference routine takes).  An unknown overburden
 * method -> CLMGB_ERR_CONFIG (the reference's error()); gridcell or landunit indices out
 * of range, or snl outside -nlevsno..0, set CLMGB_COL_PATCH_RANGE / CLMGB_COL_LEVEL_RANGE
 * in the device status and skip the column. */
int32_t clmgb_snow_layers(clmgb_handle h, const clmgb_bounds* b, const clmgb_snowlayer_fields* f,
                          const clmgb_snowlayer_config* cfg, uint32_t stages, double dtime, void* stream);

/* lake_temperature! (lake_temperature.jl:1016-1295) for the lake columns, one thread per
 * column through the whole sequence: thermal properties, eddy diffusivity, solar source,
 * the Crank-Nicolson system over snow, lake and soil levels and its tridiagonal solve,
 * phase change (phase_change_lake!), convective mixing, and the energy check that
 * moves a residual below 0.1 W/m2 into the patch's sensible heat.  Results are the
 * reference's bits.  Every pointer is required, lakeresist and grnd_ch4_cond only with
 * use_lch4.  A patch index that does not map back to its column sets
 * CLMGB_COL_PATCH_RANGE, snl outside -nlevsno..0 CLMGB_COL_LEVEL_RANGE (column skipped). */
int32_t clmgb_lake_temperature(clmgb_handle h, const clmgb_bounds* b, const clmgb_lake_fields* f,
                               const clmgb_lake_config* cfg, double dtime, void* stream);

/* soil_water! with the Zeng-Decker 2009 method (soilwater_zengdecker2009!,
 * soil_water_movement.jl:1616-1764): equilibrium matric potential from the water
 * table, one implicit tridiagonal solve over the soil layers plus the aquifer layer,
 * aquifer recharge qcharge and the water deficit.  cfg must select
 * CLMGB_ZENGDECKER_2009 with the CLMGB_BC_AQUIFER lower boundary (the reference's
 * init_soilwater_movement rejects any other pair, :681-705).  clmgb_soil_water returns
 * CLMGB_ERR_UNSUPPORTED for this method: its fields are these. */
int32_t clmgb_soil_water_zd09(clmgb_handle h, const clmgb_bounds* b, const clmgb_zd09_fields* f,
                              const clmgb_swm_config* cfg, double dtime, void* stream);

/* compute_effec_rootfrac_and_vert_tran_sink! (soil_water_plant_sink.jl:341-451) over the
 * hydrology columns: pervious roads take the transpiration-weighted root fractions
 * (the default method, which is also the roads' hydraulic-stress method, :48-78 and
 * :160-180); other columns take the default method, or with use_hydrstress the
 * soil-root conductance method (:210-245).  A column that is a pervious road on a
 * natural-vegetation landunit falls in two of the reference's filters, which then
 * raises an error: it is computed as the reference computes it and flagged
 * CLMGB_COL_FILTER. */
int32_t clmgb_effec_rootfrac_vert_tran_sink(clmgb_handle h, const clmgb_bounds* b,
                                            const clmgb_rootsink_fields* f, int32_t use_hydrstress,
                                            uint32_t* col_status, void* stream);

/* One whole column step in a single launch: t_ssbef/t_h2osfc_bef copies, soil_temperature!,
 * set_soil_water_fractions!, soil_water! (moisture form) — the driver's order
 * (clm_driver.jl:1801, 1935, 2049) when nothing runs in between.  t_ssbef and
 * t_h2osfc_bef may be NULL. */
int32_t clmgb_column_step(clmgb_handle h, const clmgb_bounds* b,
                          const clmgb_soiltemp_fields* ft, const clmgb_soilwater_fields* fw,
                          const clmgb_swm_config* cfg, double dtime, int32_t snow_method,
                          double* t_ssbef, double* t_h2osfc_bef,
                          uint32_t* col_status, void* stream);

/* soil_water! (moisture form) for callers that cannot allocate GPU memory (a host
 * runtime that owns the device memory pool, code inside stream capture, allocator-free
 * embedded callers).  No counterpart in the reference: it is the same solve as
 * clmgb_soil_water, without a handle.  It calls no cudaMalloc/cudaFree; its scratch
 * is a static device array of 16 bytes plus 4 bytes per column that every GPU
 * loading this library keeps until exit, so nc is limited to
 * CLMGB_NOALLOC_MAX_COLUMNS (larger -> CLMGB_ERR_DIMS).  All calls share that array:
 * calls that overlap on the GPU race, so issue them in order on one stream.  Each
 * call looks up the array's address in the current context; the first call on a
 * device also loads the library's module there, so make it before any stream
 * capture.  col_status (optional, device [nc]) receives the per-column status; there
 * is no accumulated device status word. */
#define CLMGB_NOALLOC_MAX_COLUMNS (1 << 20)
int32_t clmgb_soil_water_noalloc(const clmgb_varpar* vp, const clmgb_bounds* b,
                                 const clmgb_soilwater_fields* f, const clmgb_swm_config* cfg,
                                 double dtime, uint32_t* col_status, void* stream);

/* ---- component entry points (the reference exposes these functions too) ---- */

/* phase_change_h2osfc! (soil_temperature.jl:1857) and phase_change_beta!
 * (soil_temperature.jl:2232) on their own; dhsdT is a device [nc] array. */
int32_t clmgb_phase_change_h2osfc(clmgb_handle h, const clmgb_bounds* b,
                                  const clmgb_soiltemp_fields* f, double dtime,
                                  const double* dhsdT, void* stream);
int32_t clmgb_phase_change_beta(clmgb_handle h, const clmgb_bounds* b,
                                const clmgb_soiltemp_fields* f, double dtime,
                                const double* dhsdT, void* stream);

/* ---- synthetic per-step forcing (benchmark and test harness) ----
 * Stands in for the upstream modules that write the path's inputs each step
 * (radiation, infiltration; out of scope): per non-lake column, for its patches
 * sabg = sabg_soil = sabg_snow = G[c], sabg_lyr = G[c] on the top active layer and 0
 * elsewhere; forc_lwrad[c] = SB*t_grnd[c]^4; qflx_infl[c] = I[c]. */
int32_t clmgb_synth_forcing(clmgb_handle h, const clmgb_bounds* b,
                            const clmgb_soiltemp_fields* ft, const clmgb_soilwater_fields* fw,
                            const double* G, const double* I, void* stream);

/* ---- solver entry points ---- */

/* batched_band_solve! (band_diagonal.jl:179): bmatrix is [ldc, nband, nlev] (nband =
 * kl+ku+1 = 5, row-oriented bands: band b of row r is A[r, r+3-b]); rvector/tvector
 * are [ldc, nlev]; jtop/jbot int64 [nc] in the -nlevsno_off.. level numbering, the
 * solved rows are jtop+nlevsno_off+1 .. jbot+nlevsno_off+1 (1-based). */
int32_t clmgb_batched_band_solve(clmgb_handle h, int64_t nc, int64_t ldc, int32_t nlev,
                                 double* tvector, const double* bmatrix, const double* rvector,
                                 const int64_t* jtop, const int64_t* jbot, const uint8_t* mask,
                                 int32_t kl, int32_t ku, int32_t nlevsno_off, void* stream);

/* tridiagonal_multi! (tridiagonal.jl:129): a,b,c,r,u are [ldc, nlevs]; jtop int64 [nc]
 * 1-based; nlevs <= 64.  CLMGB_OPT_TRIDIAG_METHOD selects the solver: Thomas, one thread
 * per column, with the reference's 1e-30 pivot guard (CLMGB_TRIDIAG_THOMAS, the default:
 * the reference's bits), or parallel cyclic reduction, one warp per column
 * (CLMGB_TRIDIAG_PCR: log2 rounds instead of a sequential sweep, the same guard on its
 * divisors, no pivoting; for diagonally dominant systems; rounding differs from the
 * reference's in the last bits). */
int32_t clmgb_tridiagonal_multi(clmgb_handle h, int64_t ncols, int64_t ldc, int32_t nlevs,
                                double* u, const double* a, const double* b, const double* c,
                                const double* r, const int64_t* jtop, const uint8_t* mask,
                                void* stream);

/* ---- reverse-mode rules of the solves (enzyme_rules.jl) ---- */

/* The forward of batched_band_solve! that also keeps its factorisation for the
 * reverse pass (the augmented primal of the band_solve! rule, enzyme_rules.jl:80-89).
 * tvector is bit-identical to clmgb_batched_band_solve.  lu is [ldc, W, nlev] doubles,
 * W = 2*kl+ku+1 (row i of a column's system, at level jt+i, holds A's factor entries
 * U(i, i..i+kl+ku) and the multipliers of the eliminations it received); piv is
 * [ldc, nlev] bytes (row exchange of elimination step k as an offset 0..kl). */
int32_t clmgb_batched_band_solve_factor(clmgb_handle h, int64_t nc, int64_t ldc, int32_t nlev,
                                        double* tvector, const double* bmatrix, const double* rvector,
                                        const int64_t* jtop, const int64_t* jbot, const uint8_t* mask,
                                        int32_t kl, int32_t ku, int32_t nlevsno_off, double* lu,
                                        uint8_t* piv, void* stream);

/* band_solve! reverse rule (enzyme_rules.jl:91-107) over the batched layout:
 * A^T lambda = tvector_bar solved from the stored factors (LAPACK gbtrs 'T' order),
 * rvector_bar += lambda, bmatrix_bar -= lambda x^T on the band entries the forward
 * read, tvector_bar consumed (zeroed) over the solved rows.  bmatrix_bar and
 * rvector_bar may be NULL (inactive). */
int32_t clmgb_batched_band_solve_adjoint(clmgb_handle h, int64_t nc, int64_t ldc, int32_t nlev,
                                         const double* tvector, double* tvector_bar, const double* lu,
                                         const uint8_t* piv, double* bmatrix_bar, double* rvector_bar,
                                         const int64_t* jtop, const int64_t* jbot, const uint8_t* mask,
                                         int32_t kl, int32_t ku, int32_t nlevsno_off, void* stream);

/* tridiagonal_solve! reverse rule (enzyme_rules.jl:160-201) per column of the
 * [ldc, nlevs] layout, system jtop..nlevs: lambda = A^-T u_bar by the same Thomas
 * sweep on the transposed bands, r_bar += lambda, b_bar -= lambda*u,
 * a_bar[j] -= lambda[j]*u[j-1] (j > jtop), c_bar[j] -= lambda[j]*u[j+1] (j < nlevs),
 * u_bar consumed.  a_bar, b_bar, c_bar, r_bar may be NULL (inactive). */
int32_t clmgb_tridiagonal_adjoint(clmgb_handle h, int64_t ncols, int64_t ldc, int32_t nlevs,
                                  const double* u, const double* a, const double* b, const double* c,
                                  double* u_bar, double* a_bar, double* b_bar, double* c_bar,
                                  double* r_bar, const int64_t* jtop, const uint8_t* mask, void* stream);

/* ---- reverse mode through a whole column step ---- */

/* Adjoints of one column step (clmgb_column_step), all device pointers in the
 * layouts of the fields they belong to.  lam_* hold, on entry, the adjoints of the
 * step's OUTPUTS (the state after the step) and, on return, the adjoints of its
 * INPUTS (the state before it): the adjoint threaded backwards through a trajectory
 * as _reverse_step_into! (canopy_fluxes_reverse.jl:447-465) threads Enzyme's shadow.
 * lam_qcharge (may be NULL) is the adjoint of the step's qcharge output.  grad_*
 * ([ldc, nlevsoi], may be NULL) accumulate (+=) the adjoints of the hydraulic
 * parameters watsat, bsw, sucsat, hksat of levels 1..nlevsoi.  Levels above the top
 * active snow layer are left unchanged (the step does not touch them). */
typedef struct clmgb_step_adjoint {
  int64_t struct_size;               /* sizeof(clmgb_step_adjoint) */
  double* lam_t_soisno;              /* [ldc, nlevsno+nlevmaxurbgrnd] */
  double* lam_h2osoi_liq;            /* [ldc, nlevsno+nlevmaxurbgrnd] */
  double* lam_h2osoi_ice;            /* [ldc, nlevsno+nlevmaxurbgrnd] */
  double* lam_t_grnd;                /* [nc] */
  double* lam_t_h2osfc;              /* [nc] */
  const double* lam_qcharge;         /* [nc] */
  double* grad_watsat;               /* [ldc, nlevsoi] */
  double* grad_bsw;
  double* grad_sucsat;
  double* grad_hksat;
  double* lam_forc_lwrad;            /* [nc] out (may be NULL): adjoint of the step's forc_lwrad input,
                                        for callers whose forcing depends on the state */
} clmgb_step_adjoint;

/* Reserves the tape of clmgb_column_step_vjp: `slots` columns in flight (rounded up
 * to a multiple of 64) with room for `entries` recorded operations each, plus the
 * liquid-water checkpoints of up to CLMGB_ADJ_MAX_SUBSTEPS accepted Richards substeps
 * per column: slots*(entries*32 + CLMGB_ADJ_MAX_SUBSTEPS*(CLMGB_MAX_NLEVSOI+2)*8) bytes.
 * The tape holds soil_temperature! and one substep at a time (a few thousand entries
 * per column).  Synchronises the device.  A column needing more is flagged
 * CLMGB_COL_TAPE_FULL. */
#define CLMGB_ADJ_MAX_SUBSTEPS 128
int32_t clmgb_reserve_adjoint(clmgb_handle h, int64_t slots, int64_t entries);

/* Reverse of one clmgb_column_step from the state it starts from (the fields hold
 * the step's input state): replays the step (the state is left holding the step's
 * output, as the forward call leaves it, bit for bit) and propagates adj (see
 * clmgb_step_adjoint).  Needs clmgb_reserve_adjoint.  col_status gets the step's
 * status bits plus CLMGB_COL_ADJ_UNSUPPORTED / CLMGB_COL_TAPE_FULL. */
int32_t clmgb_column_step_vjp(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                              const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg,
                              double dtime, int32_t snow_method, double* t_ssbef,
                              double* t_h2osfc_bef, const clmgb_step_adjoint* adj,
                              uint32_t* col_status, void* stream);

/* Substep log of the moisture-form solve: what the reverse of a step needs from its
 * forward Richards solve, written by clmgb_column_step_logged and read by
 * clmgb_column_step_vjp_logged, so that the reverse does not run the substep loop
 * again.  rec holds, per column c, CLMGB_LOG_STRIDE(cap) doubles at
 * rec + c*CLMGB_LOG_STRIDE(cap): up to cap records of CLMGB_LOG_REC doubles (the
 * liquid water of levels 1..CLMGB_MAX_NLEVSOI at the start of an accepted substep,
 * its dtsub, the time done before it), then CLMGB_LOG_FIN doubles of the solve's
 * outputs (final liquid water, smp_l, hk_l, qcharge, attempts, status).  count[c]
 * (int32, [nc]) gets the accepted substeps, -1 for a column that was not solved; a
 * column with more than cap is reversed by running its substep loop again.
 * st_rec, when given, gets per column c CLMGB_LOG_ST_STRIDE doubles at
 * st_rec + c*CLMGB_LOG_ST_STRIDE of soil_temperature!: the factorisation of its band
 * system (factors, row exchanges, solution) and the column state the call left
 * (temperature, liquid water, ice, fact, t_grnd, t_h2osfc, status); the reverse then
 * does not run soil_temperature! again either.  Results are the same bits with or
 * without it.  No counterpart in the reference (Enzyme keeps its own tape).
 * struct_size may also be the size without the appended st_rec member. */
#define CLMGB_LOG_REC (CLMGB_MAX_NLEVSOI + 2)
#define CLMGB_LOG_FIN (3 * CLMGB_MAX_NLEVSOI + 3)
#define CLMGB_LOG_STRIDE(cap) ((int64_t)(cap) * CLMGB_LOG_REC + CLMGB_LOG_FIN)
#define CLMGB_LOG_ST_STRIDE 464
typedef struct clmgb_substep_log {
  int64_t struct_size;               /* sizeof(clmgb_substep_log) */
  double* rec;                       /* [nc * CLMGB_LOG_STRIDE(cap)] */
  int32_t* count;                    /* [nc] */
  int32_t cap;                       /* records per column, 1..CLMGB_ADJ_MAX_SUBSTEPS */
  double* st_rec;                    /* [nc * CLMGB_LOG_ST_STRIDE] or NULL */
} clmgb_substep_log;

/* clmgb_column_step that also writes the substep log (the Richards solve runs on the
 * work-queue schedule whatever CLMGB_OPT_STEP_SCHEDULE says; results are the same
 * bits). */
int32_t clmgb_column_step_logged(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                                 const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg, double dtime,
                                 int32_t snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                 const clmgb_substep_log* log, uint32_t* col_status, void* stream);

/* clmgb_column_step_vjp taking the substep log the forward step wrote from the same
 * input state (log may be NULL: the same as clmgb_column_step_vjp).  The
 * recording kernels (CLMGB_ADJ_*_RECORDED) do not read the log. */
int32_t clmgb_column_step_vjp_logged(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                                     const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg, double dtime,
                                     int32_t snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                     const clmgb_step_adjoint* adj, const clmgb_substep_log* log,
                                     uint32_t* col_status, void* stream);

/* ---- learned warm start of the moisture-form solve ----
 * A 64 -> 128 -> 128 -> 21 perceptron (SiLU hidden layers, BF16 weights and
 * activations, FP32 accumulation) proposes the size of the first substep of every
 * column: output 0 is the number k of halvings of the remaining time the solver's
 * error test needs, outputs 1..20 the saturation increment of that substep per
 * level.  Weights of a layer are [out x in] row-major BF16 (uint16_t), the last
 * layer padded to 32 outputs; feature rows are 64 BF16 values. */

/* soil_water! (moisture form) starting every column with the proposed first
 * substep dt_first[c] (clamped to [dtmin, dtime]; NaN = dtime) instead of dtime.
 * The error test accepts or halves it as any substep, so results meet the same
 * tolerance; they differ from clmgb_soil_water's by the changed substep sequence.
 * Always uses the work-queue schedule. */
int32_t clmgb_soil_water_warm(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                              const clmgb_swm_config* cfg, double dtime, const double* dt_first,
                              uint32_t* col_status, void* stream);

/* The plain solve (advances the state like clmgb_soil_water) that also records
 * training pairs at the first `per_column` substep starts of every column: 64 fp32
 * features and 32 fp32 targets per pair (target 0 = smallest k for which an attempt
 * at remaining/2^k is accepted, 1..20 = that attempt's saturation increment, the
 * rest 0), appended at rows atomically counted in *count (capacity rows at most). */
int32_t clmgb_mlp_samples(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                          const clmgb_swm_config* cfg, double dtime, int32_t per_column, float* features,
                          float* targets, uint32_t* count, int64_t capacity, uint32_t* col_status,
                          void* stream);

/* Y = act(X W^T + bias) on the tensor cores (mma.sync bf16 -> fp32): X [M x K] BF16,
 * W [N x K] BF16, bias [N] fp32 (may be NULL), act 1 = SiLU; Z [M x N] fp32
 * pre-activation and Y [M x N] BF16 are each optional.  (K, N) in {(64,128),
 * (128,128), (128,32), (32,128)}. */
int32_t clmgb_mlp_linear(clmgb_handle h, int64_t M, int32_t N, int32_t K, const uint16_t* X, int64_t ldx,
                         const uint16_t* W, const float* bias, int32_t act, float* Z, int64_t ldz,
                         uint16_t* Y, int64_t ldy, void* stream);

/* dW [N x K] += dZ^T X and db [N] += column sums of dZ (fp32 accumulation); dZ
 * [M x N] and X [M x K] BF16.  (N, K) in {(128,64), (128,128), (32,128)}. */
int32_t clmgb_mlp_linear_dw(clmgb_handle h, int64_t M, int32_t N, int32_t K, const uint16_t* dZ, int64_t lddz,
                            const uint16_t* X, int64_t ldx, float* dW, float* db, void* stream);

/* dZ = dY * silu'(Z) elementwise (n values; Z fp32, dY and dZ BF16). */
int32_t clmgb_mlp_silu_backward(clmgb_handle h, int64_t n, const float* Z, const uint16_t* dY, uint16_t* dZ,
                                void* stream);

/* loss += sum_m [w_dt (y0-t0)^2 + w_incr/20 sum_{j=1..20} (yj-tj)^2] / M over rows of
 * 32 fp32 outputs Y and targets T; dY [M x 32] BF16 its gradient. */
int32_t clmgb_mlp_loss(clmgb_handle h, int64_t M, const float* Y, const float* T, float w_dt, float w_incr,
                       float* loss, uint16_t* dY, void* stream);

/* One Adam step (bias-corrected, step >= 1) on fp32 master weights [rows x cols];
 * also writes their BF16 copy and its transpose (each may be NULL). */
int32_t clmgb_mlp_adam(clmgb_handle h, int64_t rows, int64_t cols, float* w, const float* grad, float* m,
                       float* v, float lr, float beta1, float beta2, float eps, int32_t step,
                       uint16_t* w_bf16, uint16_t* wt_bf16, void* stream);

/* Normalised BF16 features [nc x 64] of every column at the start of a solve
 * ((x - mean) * istd per feature). */
int32_t clmgb_mlp_features(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                           const clmgb_swm_config* cfg, double dtime, const float* mean, const float* istd,
                           uint16_t* X, void* stream);

/* dt_first[c] = dtime / 2^k with k = clamp(ceil(Y[c*32] - margin), 0, kmax). */
int32_t clmgb_mlp_first_dt(clmgb_handle h, int64_t nc, const float* Y, double dtime, float margin, int32_t kmax,
                           double* dt_first, void* stream);

/* ---- balance residuals (soil_fluxes.jl:321-447, balance_check.jl:741-768) ----
 * Before a step: t_grnd0[c] = t_grnd[c] and begwb[c] = the column's water (liquid +
 * ice of the active snow and ground levels, h2osfc, h2osno_no_layers). */
int32_t clmgb_balance_begin(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                            double* t_grnd0, double* begwb, void* stream);

/* After a step (t_ssbef / t_h2osfc_bef as the step saved them): the soil energy
 * residual errsoi[c] (W/m2: the ground heat flux linearised around t_grnd0 minus the
 * latent heat and the storage change of the snow and soil levels) and the water
 * residual errh2o[c] (mm: storage change minus (qflx_infl - sum qflx_rootsoi -
 * qcharge) dtime).  Urban and lake columns get 0. */
int32_t clmgb_balance_residuals(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                                const clmgb_soilwater_fields* fw, double dtime, const double* t_ssbef,
                                const double* t_h2osfc_bef, const double* t_grnd0, const double* begwb,
                                double* errsoi, double* errh2o, void* stream);

/* ---- balance_check!'s column checks (balance_check.jl:707-768, 1099-1160, 1347-1365) ---- */
/* Every field of the column water-balance check, and the soil energy residual. */
typedef struct clmgb_colbalance_fields {
  int64_t struct_size;                /* sizeof(clmgb_colbalance_fields) */
  const int64_t* col_itype;           /* [nc]  walls take no precipitation */
  const uint8_t* col_active;          /* [nc] */
  const double* forc_rain;            /* [nc]  column rain (mm/s) */
  const double* forc_snow;            /* [nc]  column snow (mm/s) */
  const double* begwb;                /* [nc]  water at the start of the step (mm) */
  const double* endwb;                /* [nc]  water at its end (mm) */
  const double* qflx_flood;           /* [nc]  mm/s, like every flux below */
  const double* qflx_sfc_irrig;       /* [nc] */
  const double* qflx_glcice_dyn_water_flux; /* [nc] */
  const double* qflx_evap_tot;        /* [nc] */
  const double* qflx_surf;            /* [nc] */
  const double* qflx_qrgwl;           /* [nc] */
  const double* qflx_drain;           /* [nc] */
  const double* qflx_drain_perched;   /* [nc] */
  const double* qflx_ice_runoff;      /* [nc] */
  const double* qflx_snwcp_discarded_liq; /* [nc] */
  const double* qflx_snwcp_discarded_ice; /* [nc] */
  const double* errsoi;               /* [nc]  soil energy residual (W/m2), e.g. from clmgb_soil_fluxes */
  double* errh2o;                     /* [nc]  W: column water residual (mm) */
} clmgb_colbalance_fields;

/* What the reference's host-side scans look at, computed on the device. */
typedef struct clmgb_balance_report {
  double  errh2o_max;                 /* maximum |errh2o| over the columns (NaN if any is NaN) */
  int64_t errh2o_index;               /* 1-based column of its first occurrence (0: no columns) */
  int64_t errh2o_nonfinite;           /* 1-based first column with a NaN/Inf errh2o (0: none) */
  double  errsoi_max;                 /* maximum |errsoi| over the active columns (0 for inactive) */
  int64_t errsoi_index;               /* 1-based column of its first occurrence */
  uint32_t flags;                     /* CLMGB_BAL_* */
  uint32_t reserved;
} clmgb_balance_report;
#define CLMGB_BAL_H2O_WARN       1u   /* errh2o_max > H2O_WARNING_THRESH (1e-9 mm), :711 */
#define CLMGB_BAL_H2O_ERROR      2u   /* errh2o_max > BALANCE_ERROR_THRESH (1e-5 mm), :713 */
#define CLMGB_BAL_H2O_NONFINITE  4u   /* some errh2o is NaN/Inf (a failure, not a pass) */
#define CLMGB_BAL_SOI_WARN       8u   /* errsoi_max > 1e-5 W/m2, :1352 */
#define CLMGB_BAL_SOI_ERROR     16u   /* errsoi_max > 1e-4 W/m2, :1356 */

/* The column part of balance_check!: errh2o (_bc_forc_rainsnow_kernel! and
 * _bc_errh2o_col_kernel!, :723-770) and the maxima and first indices its warn/error scans
 * read (:1124-1160, :1347-1365), reduced on the device.  The report is written to host
 * memory, so the call waits for `stream`.  Whether a flagged error stops the model
 * (hard_error, skip_steps, DAnstep) stays with the caller, as in the reference. */
int32_t clmgb_balance_check_columns(clmgb_handle h, const clmgb_bounds* b, const clmgb_colbalance_fields* f,
                                    double dtime, clmgb_balance_report* report, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CLMGB_H */
