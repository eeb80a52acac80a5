# CLMGB300Ext — CLM.jl package extension that routes the soil/snow column solve of
# CuArray-backed state to the GB300 kernels in libclmgb.so (include/clmgb.h).
#
# Untested in this build environment (no Julia); it is written to the C header's
# struct member order, which tests/test_abi.py pins for the Python mirror.
module CLMGB300Ext

using CLM
using CUDA

const lib = get(ENV, "CLMGB_LIB", "libclmgb.so")

struct Varpar
    nlevsno::Int32; nlevgrnd::Int32; nlevsoi::Int32; nlevurb::Int32; nlevmaxurbgrnd::Int32; reserved::Int32
end
struct Bounds
    nc::Int64; np::Int64; nl::Int64; ldc::Int64; ldp::Int64
end
struct SwmConfig
    soilwater_movement_method::Int32; upper_boundary_condition::Int32
    lower_boundary_condition::Int32; flux_calculation::Int32
    dtmin::Float64; verySmall::Float64; xTolerUpper::Float64; xTolerLower::Float64; e_ice::Float64
end

ptr(x::CuArray) = reinterpret(Ptr{Cvoid}, pointer(x))
strerror(rc) = unsafe_string(ccall((:clmgb_strerror, lib), Cstring, (Int32,), rc))
check(rc, what) = rc == 0 || error(what, ": ", strerror(rc))

const HANDLE = Ref{Ptr{Cvoid}}(C_NULL)
function handle()
    if HANDLE[] == C_NULL
        vp = Varpar(CLM.varpar.nlevsno, CLM.varpar.nlevgrnd, CLM.varpar.nlevsoi,
                    CLM.varpar.nlevurb, CLM.varpar.nlevmaxurbgrnd, 0)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:clmgb_create, lib), Int32, (Ref{Varpar}, Ref{Ptr{Cvoid}}), vp, h), "clmgb_create")
        HANDLE[] = h[]
    end
    HANDLE[]
end

# clmgb_soiltemp_fields: struct_size followed by the pointers, in header order.
function soiltemp_fields(col, lun, patch, temp, ef, ss, wsb, wdb, wfb, sa, cs, forc_lwrad,
                         mask_nolakec, mask_nolakep)
    p = Ptr{Cvoid}[
        ptr(mask_nolakec), ptr(mask_nolakep), ptr(col.snl), ptr(col.nbedrock), ptr(col.itype),
        ptr(col.landunit), ptr(col.patchi), ptr(col.patchf), ptr(lun.itype), ptr(lun.urbpoi),
        ptr(patch.column), ptr(patch.landunit), ptr(patch.wtcol), ptr(cs.frac_veg_nosno_patch),
        ptr(col.dz), ptr(col.z), ptr(col.zi),
        ptr(temp.t_soisno_col), ptr(temp.t_h2osfc_col), ptr(temp.t_grnd_col), ptr(temp.xmf_col),
        ptr(temp.xmf_h2osfc_col), ptr(temp.fact_col), ptr(temp.c_h2osfc_col), ptr(temp.imelt_col),
        ptr(temp.emg_col),
        ptr(ef.htvp_col), ptr(ef.eflx_bot_col), ptr(ef.eflx_fgr12_col), ptr(ef.eflx_fgr_col),
        ptr(ef.eflx_snomelt_col), ptr(ef.eflx_snomelt_r_col), ptr(ef.eflx_snomelt_u_col),
        ptr(ef.eflx_h2osfc_to_snow_col), ptr(ef.eflx_gnet_patch), ptr(ef.dgnetdT_patch),
        ptr(ef.dlrad_patch), ptr(ef.cgrnd_patch), ptr(ef.eflx_sh_grnd_patch), ptr(ef.eflx_sh_snow_patch),
        ptr(ef.eflx_sh_soil_patch), ptr(ef.eflx_sh_h2osfc_patch),
        ptr(ss.watsat_col), ptr(ss.bsw_col), ptr(ss.sucsat_col), ptr(ss.tkmg_col), ptr(ss.tkdry_col),
        ptr(ss.csol_col), ptr(ss.thk_col),
        ptr(wsb.ws.h2osoi_liq_col), ptr(wsb.ws.h2osoi_ice_col), ptr(wsb.ws.excess_ice_col),
        ptr(wsb.ws.h2osno_no_layers_col), ptr(wsb.ws.h2osfc_col), ptr(wsb.int_snow_col),
        ptr(wdb.frac_sno_eff_col), ptr(wdb.frac_h2osfc_col), ptr(wdb.snow_depth_col), ptr(wdb.bw_col),
        ptr(wdb.exice_subs_col), ptr(wdb.snomelt_accum_col),
        ptr(wfb.wf.qflx_evap_soi_patch), ptr(wfb.qflx_ev_snow_patch), ptr(wfb.qflx_ev_soil_patch),
        ptr(wfb.qflx_ev_h2osfc_patch), ptr(wfb.wf.qflx_snomelt_col), ptr(wfb.wf.qflx_snofrz_col),
        ptr(wfb.wf.qflx_snow_drain_col), ptr(wfb.wf.qflx_h2osfc_to_ice_col),
        ptr(wfb.wf.qflx_snomelt_lyr_col), ptr(wfb.wf.qflx_snofrz_lyr_col),
        ptr(sa.sabg_patch), ptr(sa.sabg_soil_patch), ptr(sa.sabg_snow_patch), ptr(sa.sabg_lyr_patch),
        ptr(sa.sabg_chk_patch), ptr(forc_lwrad)]
    buf = Vector{UInt8}(undef, 8 * (1 + length(p)))
    GC.@preserve buf begin
        unsafe_store!(Ptr{Int64}(pointer(buf)), Int64(length(buf)))
        for (i, q) in enumerate(p)
            unsafe_store!(Ptr{Ptr{Cvoid}}(pointer(buf) + 8i), q)
        end
    end
    buf
end

function CLM.soil_temperature!(col::CLM.ColumnData{<:Any,<:CuArray}, lun, patch, temp, ef, ss, wsb, wdb,
                               wfb, sa, cs, up, tbmax, forc_lwrad, mask_nolakec, mask_nolakep,
                               mask_urbanl, mask_urbanc, bounds_col, bounds_lun, bounds_patch, dtime;
                               urbantv_p_ac = nothing)
    f = soiltemp_fields(col, lun, patch, temp, ef, ss, wsb, wdb, wfb, sa, cs, forc_lwrad,
                        mask_nolakec, mask_nolakep)
    b = Bounds(length(bounds_col), length(bounds_patch), length(bounds_lun),
               size(temp.t_soisno_col, 1), size(sa.sabg_lyr_patch, 1))
    snow = CLM.varctl.snow_thermal_cond_method == "Jordan1991" ? Int32(1) :
           CLM.varctl.snow_thermal_cond_method == "Sturm1997" ? Int32(2) :
           error("Unknown snow_thermal_cond_method")
    GC.@preserve f begin
        check(ccall((:clmgb_soil_temperature, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Float64, Int32, Int32, Ptr{UInt32}, Ptr{Cvoid}),
                    handle(), b, f, dtime, snow, Int32(CLM.varctl.use_excess_ice), C_NULL,
                    CUDA.stream().handle), "clmgb_soil_temperature")
    end
    nothing
end

function soilwater_fields(col, mask_hydrology, sh, ss, wfb, wsb)
    p = Ptr{Cvoid}[ptr(mask_hydrology), ptr(col.nbedrock), ptr(col.dz), ptr(col.z), ptr(col.zi),
                   ptr(wsb.ws.h2osoi_liq_col), ptr(wsb.ws.h2osoi_ice_col), ptr(wsb.ws.excess_ice_col),
                   ptr(ss.watsat_col), ptr(ss.hksat_col), ptr(ss.bsw_col), ptr(ss.sucsat_col),
                   ptr(ss.eff_porosity_col), ptr(sh.icefrac_col), ptr(ss.smp_l_col), ptr(ss.hk_l_col),
                   ptr(wfb.qflx_rootsoi_col), ptr(wfb.wf.qflx_infl_col), ptr(sh.zwt_col),
                   ptr(sh.qcharge_col), ptr(sh.num_substeps_col), ptr(ss.smpmin_col)]
    buf = Vector{UInt8}(undef, 8 * (1 + length(p)))
    GC.@preserve buf begin
        unsafe_store!(Ptr{Int64}(pointer(buf)), Int64(length(buf)))
        for (i, q) in enumerate(p)
            unsafe_store!(Ptr{Ptr{Cvoid}}(pointer(buf) + 8i), q)
        end
    end
    buf
end

# a fields struct: its size, then one device pointer per member
function fields_buffer(p::Vector{Ptr{Cvoid}})
    buf = Vector{UInt8}(undef, 8 * (1 + length(p)))
    GC.@preserve buf begin
        unsafe_store!(Ptr{Int64}(pointer(buf)), Int64(length(buf)))
        for (i, q) in enumerate(p)
            unsafe_store!(Ptr{Ptr{Cvoid}}(pointer(buf) + 8i), q)
        end
    end
    buf
end

# compute_effec_rootfrac_and_vert_tran_sink! (soil_water_plant_sink.jl:341) on CuArrays
function CLM.compute_effec_rootfrac_and_vert_tran_sink!(bounds_col, nlevsoi, mask_hydrology::CuArray,
        ss, cs, wfb, ef, col, lun, patch_data; use_hydrstress::Bool = false)
    f = fields_buffer(Ptr{Cvoid}[ptr(mask_hydrology), ptr(col.itype), ptr(col.landunit), ptr(lun.itype),
                                 ptr(col.patchi), ptr(col.npatches), ptr(patch_data.active), ptr(patch_data.wtcol),
                                 ptr(ss.rootr_patch), ptr(wfb.wf.qflx_tran_veg_patch), ptr(wfb.wf.qflx_tran_veg_col),
                                 ptr(ss.rootr_col), ptr(wfb.qflx_rootsoi_col), ptr(ss.k_soil_root_patch),
                                 ptr(ss.smp_l_col), ptr(cs.vegwp_patch), ptr(cs.frac_veg_nosno_patch), ptr(col.z),
                                 ptr(wfb.qflx_phs_neg_col), ptr(wfb.qflx_hydr_redist_patch)])
    b = Bounds(length(mask_hydrology), length(patch_data.wtcol), length(lun.itype), size(col.z, 1),
               length(patch_data.wtcol))
    GC.@preserve f begin
        check(ccall((:clmgb_effec_rootfrac_vert_tran_sink, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Int32, Ptr{UInt32}, Ptr{Cvoid}),
                    handle(), b, f, Int32(use_hydrstress), C_NULL, CUDA.stream().handle),
              "clmgb_effec_rootfrac_vert_tran_sink")
    end
    nothing
end

function CLM.soil_water!(col::CLM.ColumnData{<:Any,<:CuArray}, mask_hydrology, mask_urban, sh, ss, wfb,
                         wsb, temp, cs, ef, swrc, cfg::CLM.SoilWaterMovementConfig, dtime;
                         use_flexibleCN::Bool = false)
    c = SwmConfig(cfg.soilwater_movement_method, cfg.upper_boundary_condition, cfg.lower_boundary_condition,
                  cfg.flux_calculation, cfg.dtmin, cfg.verySmall, cfg.xTolerUpper, cfg.xTolerLower, cfg.e_ice)
    b = Bounds(length(mask_hydrology), 0, 0, size(col.dz, 1), 0)
    if cfg.soilwater_movement_method == CLM.ZENGDECKER_2009
        # soilwater_zengdecker2009! has its own field set (clmgb_zd09_fields)
        z = fields_buffer(Ptr{Cvoid}[ptr(mask_hydrology), ptr(col.dz), ptr(col.z), ptr(col.zi),
                                     ptr(temp.t_soisno_col), ptr(wsb.ws.h2osoi_liq_col),
                                     ptr(wsb.ws.h2osoi_ice_col), ptr(wsb.ws.h2osoi_vol_col), ptr(ss.watsat_col),
                                     ptr(ss.hksat_col), ptr(ss.bsw_col), ptr(ss.sucsat_col), ptr(ss.smpmin_col),
                                     ptr(sh.icefrac_col), ptr(ss.smp_l_col), ptr(ss.hk_l_col),
                                     ptr(wfb.qflx_rootsoi_col), ptr(wfb.wf.qflx_infl_col), ptr(sh.zwt_col),
                                     ptr(sh.qcharge_col), ptr(wfb.qflx_deficit_col)])
        GC.@preserve z begin
            check(ccall((:clmgb_soil_water_zd09, lib), Int32,
                        (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ref{SwmConfig}, Float64, Ptr{Cvoid}),
                        handle(), b, z, c, dtime, CUDA.stream().handle), "clmgb_soil_water_zd09")
        end
        return nothing
    end
    f = soilwater_fields(col, mask_hydrology, sh, ss, wfb, wsb)
    GC.@preserve f begin
        check(ccall((:clmgb_soil_water, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ref{SwmConfig}, Float64, Ptr{UInt32}, Ptr{Cvoid}),
                    handle(), b, f, c, dtime, C_NULL, CUDA.stream().handle), "clmgb_soil_water")
    end
    use_flexibleCN && flexible_cn!(col, mask_hydrology, wsb, b)
    nothing
end

# soil_water!'s use_flexibleCN step (soil_water_movement.jl:1812-1843): clmgb_soil_water_flexible_cn
function flexible_cn!(col, mask_hydrology, wsb, b::Bounds)
    f = fields_buffer(Ptr{Cvoid}[ptr(mask_hydrology), ptr(col.dz), ptr(wsb.ws.h2osoi_liq_col),
                                 ptr(wsb.ws.h2osoi_ice_col), ptr(wsb.ws.h2osoi_vol_col), ptr(wsb.ws.wa_col)])
    GC.@preserve f begin
        check(ccall((:clmgb_soil_water_flexible_cn, lib), Int32, (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ptr{Cvoid}),
                    handle(), b, f, CUDA.stream().handle), "clmgb_soil_water_flexible_cn")
    end
    nothing
end

# ---------------------------------------------------------------------------
# Surface hydrology before soil_water! (clm_driver.jl:1938-2007): each routine is one
# stage of clmgb_surface_hydrology; the whole sequence is one call with every bit.
# Members a stage does not read stay NULL (the library checks only the selected ones).
# ---------------------------------------------------------------------------
struct SurfHydConfig
    struct_size::Int64; ng::Int64
    fsat_method::Int32; crop_fsat_equals_zero::Int32; hillslope_fsat_equals_zero::Int32
    qinmax_method::Int32; h2osfcflag::Int32; update_h2osfcflag::Int32
    fff::Float64; e_ice::Float64; pc::Float64; mu::Float64; pondmx_urban::Float64
end
const SH = (floodc = 0x1, sat_excess = 0x2, qflx_inputs = 0x4, infl_excess = 0x8, route = 0x10,
            update_h2osfc = 0x20, infiltration = 0x40, total_runoff = 0x80, urban_ponding = 0x100)
const SURFHYD_MEMBERS = (
    :mask_nolakec, :mask_hydrology, :mask_urban, :col_snl, :col_itype, :col_landunit, :col_gridcell,
    :col_urbpoi, :col_is_hillslope, :col_active, :col_cold, :lun_itype, :qflx_floodg, :frost_table, :zwt,
    :zwt_perched, :wtfact, :b_infil, :top_max_moist, :top_moist_limited, :icefrac, :hksat, :frac_sno_eff,
    :frac_h2osfc, :frac_h2osfc_nosnow, :h2osfc_thresh, :topo_slope, :qflx_rain_plus_snomelt, :qflx_snow_h2osfc,
    :qflx_liqevap_from_top_layer, :qflx_ev_soil, :qflx_ev_h2osfc, :qflx_floodc, :fsat, :fcov,
    :qflx_sat_excess_surf, :qflx_top_soil, :qflx_in_soil, :qflx_top_soil_to_h2osfc, :qinmax, :qflx_infl_excess,
    :qflx_in_soil_limited, :qflx_in_h2osfc, :qflx_infl_excess_surf, :h2osfc, :qflx_h2osfc_surf,
    :qflx_h2osfc_drain, :qflx_infl, :qflx_surf, :xs_urban, :h2osoi_liq)


surfhyd_config(; ng = 1, fsat_method = CLM.FSAT_METHOD_TOPMODEL, crop = false, hillslope = false,
               qinmax_method = CLM.QINMAX_METHOD_HKSAT, h2osfcflag = 1, update_h2osfcflag = 1) =
    SurfHydConfig(sizeof(SurfHydConfig), ng, fsat_method, crop, hillslope, qinmax_method, h2osfcflag,
                  update_h2osfcflag, CLM.sat_excess_runoff_params.fff, CLM.infilt_excess_params.e_ice,
                  CLM.SURFACE_WATER_PC[], CLM.SURFACE_WATER_MU[], CLM.PONDMX_URBAN)

function surface_hydrology!(stages, cfg::SurfHydConfig, nc, ldc, nl, dtime; arrays...)
    p = Ptr{Cvoid}[haskey(arrays, m) ? ptr(arrays[m]) : C_NULL for m in SURFHYD_MEMBERS]
    f = fields_buffer(p)
    GC.@preserve f begin
        check(ccall((:clmgb_surface_hydrology, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ref{SurfHydConfig}, UInt32, Float64, Ptr{Cvoid}),
                    handle(), Bounds(nc, 0, nl, ldc, 0), f, cfg, UInt32(stages), Float64(dtime),
                    CUDA.stream().handle), "clmgb_surface_hydrology")
    end
    nothing
end

CLM.set_floodc!(qflx_floodc, qflx_floodg, col_gridcell, col_itype, mask_nolake::CuArray, bounds) =
    surface_hydrology!(SH.floodc, surfhyd_config(ng = length(qflx_floodg)), length(mask_nolake),
                       length(mask_nolake), 1, 1.0; mask_nolakec = mask_nolake, qflx_floodg, col_gridcell,
                       col_itype, qflx_floodc)

function CLM.saturated_excess_runoff!(ser, mask_hydrology::CuArray, bounds_col, col, lun, sh, ss, wfb;
                                      crop_fsat_equals_zero::Bool = false, hillslope_fsat_equals_zero::Bool = false)
    nc = length(mask_hydrology)
    surface_hydrology!(SH.sat_excess, surfhyd_config(fsat_method = ser.fsat_method, crop = crop_fsat_equals_zero,
                                                     hillslope = hillslope_fsat_equals_zero),
                       nc, nc, length(lun.itype), 1.0; mask_hydrology, frost_table = sh.frost_table_col,
                       zwt = sh.zwt_col, zwt_perched = sh.zwt_perched_col, wtfact = ss.wtfact_col,
                       b_infil = sh.b_infil_col, top_max_moist = sh.top_max_moist_col,
                       top_moist_limited = sh.top_moist_limited_col, col_landunit = col.landunit,
                       lun_itype = lun.itype, col_is_hillslope = col.is_hillslope_column, col_active = col.active,
                       col_cold = col.cold, col_urbpoi = col.urbpoi, qflx_floodc = wfb.wf.qflx_floodc_col,
                       qflx_rain_plus_snomelt = wfb.wf.qflx_rain_plus_snomelt_col, fsat = ser.fsat_col,
                       fcov = ser.fcov_col, qflx_sat_excess_surf = wfb.qflx_sat_excess_surf_col)
end

function CLM.set_qflx_inputs!(wfb, wdb, col_snl, mask_hydrology::CuArray, bounds)
    nc = length(mask_hydrology)
    surface_hydrology!(SH.qflx_inputs, surfhyd_config(), nc, nc, 1, 1.0; mask_hydrology, col_snl,
                       qflx_rain_plus_snomelt = wfb.wf.qflx_rain_plus_snomelt_col,
                       qflx_snow_h2osfc = wfb.wf.qflx_snow_h2osfc_col, qflx_floodc = wfb.wf.qflx_floodc_col,
                       qflx_liqevap_from_top_layer = wfb.wf.qflx_liqevap_from_top_layer_col,
                       qflx_ev_soil = wfb.qflx_ev_soil_col, qflx_ev_h2osfc = wfb.qflx_ev_h2osfc_col,
                       qflx_sat_excess_surf = wfb.qflx_sat_excess_surf_col, frac_sno_eff = wdb.frac_sno_eff_col,
                       frac_h2osfc = wdb.frac_h2osfc_col, qflx_top_soil = wfb.wf.qflx_top_soil_col,
                       qflx_in_soil = wfb.qflx_in_soil_col, qflx_top_soil_to_h2osfc = wfb.qflx_top_soil_to_h2osfc_col)
end

function CLM.infiltration_excess_runoff!(ier, sh, ss, fsat_col, wfb, wdb, mask_hydrology::CuArray, bounds;
                                         params = CLM.infilt_excess_params)
    nc = length(mask_hydrology)
    cfg = surfhyd_config(qinmax_method = ier.qinmax_method)
    cfg = SurfHydConfig(cfg.struct_size, cfg.ng, cfg.fsat_method, cfg.crop_fsat_equals_zero,
                        cfg.hillslope_fsat_equals_zero, cfg.qinmax_method, cfg.h2osfcflag, cfg.update_h2osfcflag,
                        cfg.fff, params.e_ice, cfg.pc, cfg.mu, cfg.pondmx_urban)
    surface_hydrology!(SH.infl_excess, cfg, nc, size(sh.icefrac_col, 1), 1, 1.0; mask_hydrology,
                       icefrac = sh.icefrac_col, hksat = ss.hksat_col, fsat = fsat_col,
                       qflx_in_soil = wfb.qflx_in_soil_col, frac_h2osfc = wdb.frac_h2osfc_col,
                       qinmax = ier.qinmax_col, qflx_infl_excess = wfb.qflx_infl_excess_col)
end

function CLM.route_infiltration_excess!(wfb, sh, col_landunit, lun_itype, mask_hydrology::CuArray, bounds)
    nc = length(mask_hydrology)
    surface_hydrology!(SH.route, surfhyd_config(h2osfcflag = sh.h2osfcflag), nc, nc, length(lun_itype), 1.0;
                       mask_hydrology, col_landunit, lun_itype, qflx_in_soil = wfb.qflx_in_soil_col,
                       qflx_top_soil_to_h2osfc = wfb.qflx_top_soil_to_h2osfc_col,
                       qflx_infl_excess = wfb.qflx_infl_excess_col, qflx_in_soil_limited = wfb.qflx_in_soil_limited_col,
                       qflx_in_h2osfc = wfb.qflx_in_h2osfc_col, qflx_infl_excess_surf = wfb.qflx_infl_excess_surf_col)
end

function CLM.update_h2osfc!(col_data, sh, ef, wfb, wsb, wdb, mask_hydrologyc::CuArray, bounds_col;
                            dtime::Real = 1800.0, h2osfcflag::Int = 1, qinmax = nothing)
    nc = length(mask_hydrologyc)
    q = qinmax === nothing ? CUDA.zeros(Float64, nc) : qinmax
    surface_hydrology!(SH.update_h2osfc, surfhyd_config(update_h2osfcflag = h2osfcflag), nc, nc, 1, dtime;
                       mask_hydrology = mask_hydrologyc, h2osfc = wsb.ws.h2osfc_col,
                       h2osfc_thresh = sh.h2osfc_thresh_col, frac_h2osfc_nosnow = wdb.frac_h2osfc_nosnow_col,
                       topo_slope = col_data.topo_slope, qflx_in_h2osfc = wfb.qflx_in_h2osfc_col,
                       frac_h2osfc = wdb.frac_h2osfc_col, qinmax = q, qflx_h2osfc_surf = wfb.qflx_h2osfc_surf_col,
                       qflx_h2osfc_drain = wfb.qflx_h2osfc_drain_col)
end

function CLM.infiltration!(wfb, mask_hydrology::CuArray, bounds)
    nc = length(mask_hydrology)
    surface_hydrology!(SH.infiltration, surfhyd_config(), nc, nc, 1, 1.0; mask_hydrology,
                       qflx_in_soil_limited = wfb.qflx_in_soil_limited_col,
                       qflx_h2osfc_drain = wfb.qflx_h2osfc_drain_col, qflx_infl = wfb.wf.qflx_infl_col)
end

function CLM.total_surface_runoff!(wfb, sh, ws, col_snl, col_itype, col_landunit, lun_urbpoi,
                                   mask_hydrology::CuArray, mask_urban, bounds, dtime)
    nc = length(mask_hydrology)
    surface_hydrology!(SH.total_runoff, surfhyd_config(), nc, size(ws.h2osoi_liq_col, 1), 1, dtime;
                       mask_hydrology, mask_urban, col_snl, col_itype,
                       qflx_sat_excess_surf = wfb.qflx_sat_excess_surf_col,
                       qflx_infl_excess_surf = wfb.qflx_infl_excess_surf_col,
                       qflx_h2osfc_surf = wfb.qflx_h2osfc_surf_col, qflx_surf = wfb.wf.qflx_surf_col,
                       qflx_rain_plus_snomelt = wfb.wf.qflx_rain_plus_snomelt_col, h2osoi_liq = ws.h2osoi_liq_col,
                       qflx_liqevap_from_top_layer = wfb.wf.qflx_liqevap_from_top_layer_col,
                       qflx_floodc = wfb.wf.qflx_floodc_col, xs_urban = sh.xs_urban_col)
end

function CLM.update_urban_ponding!(ws, sh, wfb, col_snl, col_itype, mask_urban::CuArray, bounds, dtime)
    nc = length(mask_urban)
    surface_hydrology!(SH.urban_ponding, surfhyd_config(), nc, size(ws.h2osoi_liq_col, 1), 1, dtime;
                       mask_urban, col_snl, col_itype, xs_urban = sh.xs_urban_col,
                       qflx_rain_plus_snomelt = wfb.wf.qflx_rain_plus_snomelt_col,
                       qflx_liqevap_from_top_layer = wfb.wf.qflx_liqevap_from_top_layer_col,
                       h2osoi_liq = ws.h2osoi_liq_col)
end

# ---------------------------------------------------------------------------
# Snow layer dynamics after the soil solve (clm_driver.jl:2146-2200): each routine is one
# stage of clmgb_snow_layers (the arrays a routine does not take stay NULL).
# ---------------------------------------------------------------------------
struct SnowLayerConfig
    struct_size::Int64; ng::Int64
    use_subgrid_fluxes::Int32; overburden_method::Int32; wind_dependent_snow_density::Int32; is_lake::Int32
    int_snow_max::Float64; overburden_compress_tfactor::Float64; upplim_destruct_metamorph::Float64
    eta0_anderson::Float64; eta0_vionnet::Float64; ceta::Float64; drift_gs::Float64; rho_min::Float64
    rho_max::Float64; tau_ref::Float64; snw_rds_min::Float64; snw_rds_max::Float64
    dzmin_1::Float64; dzmin_2::Float64; dzmax_l_1::Float64; dzmax_l_2::Float64; dzmax_u_1::Float64
    dzmax_u_2::Float64
end
const SL = (compaction = 0x1, combine = 0x2, divide = 0x4, zero_empty = 0x8, filter = 0x10)
const SNOWLAYER_MEMBERS = (
    :mask_snow, :mask_nosnow, :mask_nolakec, :col_snl, :col_landunit, :col_gridcell, :lun_itype, :lun_lakpoi,
    :lun_urbpoi, :forc_wind, :n_melt, :frac_h2osfc, :frac_sno, :frac_sno_eff, :int_snow, :h2osno_no_layers,
    :snow_depth, :qflx_sl_top_soil, :dz, :z, :zi, :t_soisno, :h2osoi_ice, :h2osoi_liq, :imelt, :swe_old,
    :frac_iceold, :snw_rds, :mss_bcphi, :mss_bcpho, :mss_ocphi, :mss_ocpho, :mss_dst1, :mss_dst2, :mss_dst3,
    :mss_dst4)


function snowlayer_config(; ng = 1, is_lake = false, use_subgrid_fluxes = CLM.varctl.use_subgrid_fluxes,
                          int_snow_max = 2000.0)
    p = CLM.snowhydrology_params
    SnowLayerConfig(sizeof(SnowLayerConfig), ng, use_subgrid_fluxes, CLM.OVERBURDEN_COMPACTION_METHOD[],
                    CLM.WIND_DEPENDENT_SNOW_DENSITY[], is_lake, int_snow_max, CLM.OVERBURDEN_COMPRESS_TFACTOR[],
                    p.upplim_destruct_metamorph, p.eta0_anderson, p.eta0_vionnet, p.ceta, p.drift_gs, p.rho_min,
                    p.rho_max, p.tau_ref, p.snw_rds_min, CLM.SNW_RDS_MAX, CLM.SNOW_DZMIN_1[], CLM.SNOW_DZMIN_2[],
                    CLM.SNOW_DZMAX_L_1[], CLM.SNOW_DZMAX_L_2[], CLM.SNOW_DZMAX_U_1[], CLM.SNOW_DZMAX_U_2[])
end

function snow_layers!(stages, cfg::SnowLayerConfig, nc, ldc, nl, dtime; arrays...)
    p = Ptr{Cvoid}[haskey(arrays, m) ? ptr(arrays[m]) : C_NULL for m in SNOWLAYER_MEMBERS]
    f = fields_buffer(p)
    GC.@preserve f begin
        check(ccall((:clmgb_snow_layers, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ref{SnowLayerConfig}, UInt32, Float64, Ptr{Cvoid}),
                    handle(), Bounds(nc, 0, nl, ldc, 0), f, cfg, UInt32(stages), Float64(dtime),
                    CUDA.stream().handle), "clmgb_snow_layers")
    end
    nothing
end

aerosol_arrays(aer) = (mss_bcphi = aer.mss_bcphi_col, mss_bcpho = aer.mss_bcpho_col, mss_ocphi = aer.mss_ocphi_col,
                       mss_ocpho = aer.mss_ocpho_col, mss_dst1 = aer.mss_dst1_col, mss_dst2 = aer.mss_dst2_col,
                       mss_dst3 = aer.mss_dst3_col, mss_dst4 = aer.mss_dst4_col)

function CLM.snow_compaction!(dz::CuArray, dtime, snl, t_soisno, h2osoi_ice, h2osoi_liq, imelt, frac_sno,
                              frac_h2osfc, swe_old, int_snow, frac_iceold, forc_wind, col_gridcell, col_landunit,
                              lakpoi, urbpoi, mask_snow, bounds, nlevsno; use_subgrid_fluxes::Bool = true,
                              n_melt = CUDA.fill(20.0, length(snl)), int_snow_max::Real = 2000.0)
    nc = length(snl)
    snow_layers!(SL.compaction, snowlayer_config(ng = length(forc_wind); use_subgrid_fluxes, int_snow_max), nc,
                 size(dz, 1), length(lakpoi), dtime; mask_snow, col_snl = snl, col_landunit, col_gridcell,
                 lun_lakpoi = lakpoi, lun_urbpoi = urbpoi, forc_wind, n_melt = CuArray(Float64.(n_melt)),
                 frac_h2osfc, frac_sno, int_snow, dz, t_soisno, h2osoi_ice, h2osoi_liq, imelt, swe_old, frac_iceold)
end

function CLM.combine_snow_layers!(snl::CuArray, dz, zi, z, t_soisno, h2osoi_ice, h2osoi_liq, h2osno_no_layers,
                                  snow_depth, frac_sno, frac_sno_eff, int_snow, snw_rds, aerosol, lun_itype, urbpoi,
                                  col_landunit, mask_snow, bounds, nlevsno, qflx_sl_top_soil, dtime)
    snow_layers!(SL.combine, snowlayer_config(), length(snl), size(dz, 1), length(lun_itype), dtime;
                 mask_snow, col_snl = snl, col_landunit, lun_itype, lun_urbpoi = urbpoi, frac_sno, frac_sno_eff,
                 int_snow, h2osno_no_layers, snow_depth, qflx_sl_top_soil, dz, z, zi, t_soisno, h2osoi_ice,
                 h2osoi_liq, snw_rds, aerosol_arrays(aerosol)...)
end

function CLM.divide_snow_layers!(snl::CuArray, dz, zi, z, t_soisno, h2osoi_ice, h2osoi_liq, frac_sno, snw_rds,
                                 aerosol, is_lake::Bool, mask_snow, bounds, nlevsno)
    snow_layers!(SL.divide, snowlayer_config(; is_lake), length(snl), size(dz, 1), 1, 1.0; mask_snow, col_snl = snl,
                 frac_sno, dz, z, zi, t_soisno, h2osoi_ice, h2osoi_liq, snw_rds, aerosol_arrays(aerosol)...)
end

CLM.zero_empty_snow_layers!(snl::CuArray, dz, z, zi, t_soisno, h2osoi_ice, h2osoi_liq, mask_snow, bounds, nlevsno) =
    snow_layers!(SL.zero_empty, snowlayer_config(), length(snl), size(dz, 1), 1, 1.0; mask_snow, col_snl = snl,
                 dz, z, zi, t_soisno, h2osoi_ice, h2osoi_liq)

CLM.build_snow_filter!(mask_snow::CuArray, mask_nosnow, snl, mask_nolake, bounds) =
    snow_layers!(SL.filter, snowlayer_config(), length(snl), length(snl), 1, 1.0; mask_snow, mask_nosnow,
                 mask_nolakec = mask_nolake, col_snl = snl)

# ---------------------------------------------------------------------------
# lake_temperature! (lake_temperature.jl:1016) on CuArrays: clmgb_lake_temperature.
# ---------------------------------------------------------------------------
struct LakeConfig
    struct_size::Int64
    nlevlak::Int32; use_lch4::Int32; lakepuddling::Int32; lake_no_ed::Int32
    deepmixing_depthcrit::Float64; deepmixing_mixfact::Float64; lake_puddle_thick::Float64
end

function CLM.lake_temperature!(col::CLM.ColumnData{<:Any,<:CuArray}, patch_data, solarabs, soilstate,
                               waterstatebulk, waterdiagbulk, waterfluxbulk, energyflux, temperature, lakestate,
                               grnd_ch4_cond, mask_lakec, mask_lakep, bounds_col, bounds_patch, dtime)
    lc = CLM.lake_con
    cfg = LakeConfig(sizeof(LakeConfig), CLM.varpar.nlevlak, CLM.varctl.use_lch4, lc.lakepuddling, lc.lake_no_ed,
                     lc.deepmixing_depthcrit, lc.deepmixing_mixfact, lc.lake_puddle_thick)
    ws, wf = waterstatebulk.ws, waterfluxbulk.wf
    f = fields_buffer(Ptr{Cvoid}[
        ptr(mask_lakec), ptr(mask_lakep), ptr(col.patchi), ptr(patch_data.column), ptr(col.snl), ptr(col.dz),
        ptr(col.z), ptr(col.zi), ptr(col.dz_lake), ptr(col.z_lake), ptr(col.lakedepth), ptr(soilstate.watsat_col),
        ptr(soilstate.tksatu_col), ptr(soilstate.tkmg_col), ptr(soilstate.tkdry_col), ptr(soilstate.csol_col),
        ptr(temperature.t_grnd_col), ptr(lakestate.etal_col), ptr(lakestate.ks_col), ptr(lakestate.ws_col),
        ptr(lakestate.lake_raw_col), ptr(temperature.t_soisno_col), ptr(temperature.t_lake_col),
        ptr(ws.h2osoi_liq_col), ptr(ws.h2osoi_ice_col), ptr(ws.h2osno_no_layers_col),
        ptr(waterdiagbulk.snow_depth_col), ptr(waterdiagbulk.frac_iceold_col), ptr(lakestate.betaprime_col),
        ptr(lakestate.lake_icefrac_col), ptr(lakestate.lake_icefracsurf_col), ptr(lakestate.lake_icethick_col),
        ptr(lakestate.savedtke1_col), ptr(lakestate.lakeresist_col), ptr(grnd_ch4_cond), ptr(wf.qflx_snomelt_col),
        ptr(wf.qflx_snofrz_col), ptr(wf.qflx_snow_drain_col), ptr(wf.qflx_snomelt_lyr_col),
        ptr(wf.qflx_snofrz_lyr_col), ptr(temperature.imelt_col), ptr(energyflux.eflx_snomelt_col),
        ptr(energyflux.errsoi_col), ptr(solarabs.sabg_patch), ptr(solarabs.sabg_lyr_patch),
        ptr(solarabs.fsds_nir_d_patch), ptr(solarabs.fsds_nir_i_patch), ptr(solarabs.fsr_nir_d_patch),
        ptr(solarabs.fsr_nir_i_patch), ptr(energyflux.eflx_gnet_patch), ptr(energyflux.eflx_sh_tot_patch),
        ptr(energyflux.eflx_sh_grnd_patch), ptr(energyflux.eflx_soil_grnd_patch)])
    b = Bounds(length(mask_lakec), length(mask_lakep), 1, size(col.dz, 1), size(solarabs.sabg_lyr_patch, 1))
    GC.@preserve f begin
        check(ccall((:clmgb_lake_temperature, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ref{LakeConfig}, Float64, Ptr{Cvoid}),
                    handle(), b, f, cfg, dtime, CUDA.stream().handle), "clmgb_lake_temperature")
    end
    nothing
end

# ---------------------------------------------------------------------------
# balance_check!'s column part on CuArrays (balance_check.jl:1099-1160, 1347-1365): errh2o
# and the scans' maxima computed on the device; the stop decision stays in balance_check!
# (hard_error, skip_steps), which calls this for its CuArray columns and applies it.
# ---------------------------------------------------------------------------
struct BalanceReport
    errh2o_max::Float64; errh2o_index::Int64; errh2o_nonfinite::Int64
    errsoi_max::Float64; errsoi_index::Int64; flags::UInt32; reserved::UInt32
end

function column_balance_check!(errh2o::CuArray, col, wb, wf, wfb, forc_rain_col, forc_snow_col, qflx_ice_runoff_col,
                               errsoi_col, dtime)
    f = fields_buffer(Ptr{Cvoid}[
        ptr(col.itype), ptr(col.active), ptr(forc_rain_col), ptr(forc_snow_col), ptr(wb.begwb_col), ptr(wb.endwb_col),
        ptr(wf.qflx_floodc_col), ptr(wf.qflx_sfc_irrig_col), ptr(wf.qflx_glcice_dyn_water_flux_col),
        ptr(wf.qflx_evap_tot_col), ptr(wf.qflx_surf_col), ptr(wf.qflx_qrgwl_col), ptr(wf.qflx_drain_col),
        ptr(wf.qflx_drain_perched_col), ptr(qflx_ice_runoff_col), ptr(wf.qflx_snwcp_discarded_liq_col),
        ptr(wf.qflx_snwcp_discarded_ice_col), ptr(errsoi_col), ptr(errh2o)])
    rep = Ref{BalanceReport}()
    GC.@preserve f begin
        check(ccall((:clmgb_balance_check_columns, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Float64, Ref{BalanceReport}, Ptr{Cvoid}),
                    handle(), Bounds(length(errh2o), 0, 0, length(errh2o), 0), f, dtime, rep,
                    CUDA.stream().handle), "clmgb_balance_check_columns")
    end
    rep[]
end

# ---------------------------------------------------------------------------
# The batched solvers on CuArrays: batched_band_solve! (band_diagonal.jl:179) and
# tridiagonal_multi! (tridiagonal.jl:129), and the pieces of their reverse rules
# (CLMGB300ADExt): the forward that keeps its factorisation and the two adjoints.
# jtop/jbot are the reference's Int vectors, mask its Bool vector (a CuArray{Bool} is
# one byte per element).
# ---------------------------------------------------------------------------
function CLM.batched_band_solve!(tvector::CuArray{Float64,2}, bmatrix, rvector, jtop, jbot, mask,
                                 kl::Int, ku::Int, nlevsno_off::Int)
    nc, nlev = size(tvector)
    check(ccall((:clmgb_batched_band_solve, lib), Int32,
                (Ptr{Cvoid}, Int64, Int64, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Cvoid}, Int32, Int32, Int32, Ptr{Cvoid}),
                handle(), nc, nc, nlev, ptr(tvector), ptr(bmatrix), ptr(rvector), ptr(jtop), ptr(jbot), ptr(mask),
                kl, ku, nlevsno_off, CUDA.stream().handle), "clmgb_batched_band_solve")
    nothing
end

function band_factor_solve!(tvector::CuArray{Float64,2}, bmatrix, rvector, jtop, jbot, mask, kl, ku, nlevsno_off,
                            lu::CuArray{Float64,3}, piv::CuArray{UInt8,2})
    nc, nlev = size(tvector)
    check(ccall((:clmgb_batched_band_solve_factor, lib), Int32,
                (Ptr{Cvoid}, Int64, Int64, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Cvoid}, Int32, Int32, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                handle(), nc, nc, nlev, ptr(tvector), ptr(bmatrix), ptr(rvector), ptr(jtop), ptr(jbot), ptr(mask),
                kl, ku, nlevsno_off, ptr(lu), ptr(piv), CUDA.stream().handle), "clmgb_batched_band_solve_factor")
    nothing
end

optptr(x) = x === nothing ? C_NULL : ptr(x)

# lambda = A^-T tbar from the kept factors; rbar += lambda, bbar -= lambda x^T (band entries
# the forward read); tbar consumed.  bbar / rbar may be `nothing` (inactive).
function band_solve_adjoint!(x::CuArray{Float64,2}, tbar, lu, piv, bbar, rbar, jtop, jbot, mask, kl, ku, nlevsno_off)
    nc, nlev = size(x)
    check(ccall((:clmgb_batched_band_solve_adjoint, lib), Int32,
                (Ptr{Cvoid}, Int64, Int64, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int32, Int32, Int32, Ptr{Cvoid}),
                handle(), nc, nc, nlev, ptr(x), ptr(tbar), ptr(lu), ptr(piv), optptr(bbar), optptr(rbar), ptr(jtop),
                ptr(jbot), ptr(mask), kl, ku, nlevsno_off, CUDA.stream().handle), "clmgb_batched_band_solve_adjoint")
    nothing
end

function CLM.tridiagonal_multi!(u::CuArray{Float64,2}, a, b, c, r, jtop, mask, ncols::Int, nlevs::Int)
    check(ccall((:clmgb_tridiagonal_multi, lib), Int32,
                (Ptr{Cvoid}, Int64, Int64, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                handle(), ncols, size(u, 1), nlevs, ptr(u), ptr(a), ptr(b), ptr(c), ptr(r), ptr(jtop), ptr(mask),
                CUDA.stream().handle), "clmgb_tridiagonal_multi")
    nothing
end

# enzyme_rules.jl:160-201 per column: lambda = A^-T ubar by Thomas on the transposed bands,
# rbar += lambda, bbar -= lambda u, abar -= lambda u[j-1], cbar -= lambda u[j+1]; ubar consumed.
function tridiagonal_adjoint!(u::CuArray{Float64,2}, a, b, c, ubar, abar, bbar, cbar, rbar, jtop, mask,
                              ncols::Int, nlevs::Int)
    check(ccall((:clmgb_tridiagonal_adjoint, lib), Int32,
                (Ptr{Cvoid}, Int64, Int64, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                handle(), ncols, size(u, 1), nlevs, ptr(u), ptr(a), ptr(b), ptr(c), ptr(ubar), optptr(abar),
                optptr(bbar), optptr(cbar), optptr(rbar), ptr(jtop), ptr(mask), CUDA.stream().handle),
          "clmgb_tridiagonal_adjoint")
    nothing
end

# ---------------------------------------------------------------------------
# Reverse mode.  One column step's vector-Jacobian product (clmgb_column_step_vjp)
# behind a ChainRulesCore.rrule and an Enzyme reverse rule, the counterparts of the
# reference's _reverse_step_into! (canopy_fluxes_reverse.jl:447-465).  `StepState`
# bundles the CuArray fields of the step; its pullback maps the adjoints of the
# step's outputs to those of its inputs and of the hydraulic parameters.
# ---------------------------------------------------------------------------
struct StepAdjoint
    struct_size::Int64
    lam_t_soisno::Ptr{Cvoid}; lam_h2osoi_liq::Ptr{Cvoid}; lam_h2osoi_ice::Ptr{Cvoid}
    lam_t_grnd::Ptr{Cvoid}; lam_t_h2osfc::Ptr{Cvoid}; lam_qcharge::Ptr{Cvoid}
    grad_watsat::Ptr{Cvoid}; grad_bsw::Ptr{Cvoid}; grad_sucsat::Ptr{Cvoid}; grad_hksat::Ptr{Cvoid}
    lam_forc_lwrad::Ptr{Cvoid}
end

const TAPE_RESERVED = Ref(false)
function reserve_adjoint!(slots::Integer, entries::Integer = 8192)
    check(ccall((:clmgb_reserve_adjoint, lib), Int32, (Ptr{Cvoid}, Int64, Int64), handle(), slots, entries),
          "clmgb_reserve_adjoint")
    TAPE_RESERVED[] = true
end

# lam: NamedTuple of CuArrays (t_soisno, h2osoi_liq, h2osoi_ice, t_grnd, t_h2osfc,
# qcharge, forc_lwrad) in the fields' layouts; grad: (watsat, bsw, sucsat, hksat),
# each [nc, nlevsoi], accumulated.
function column_step_vjp!(ft_buf, fw_buf, b::Bounds, cfg::SwmConfig, dtime, snow_method, t_ssbef, t_h2osfc_bef,
                          lam, grad)
    TAPE_RESERVED[] || reserve_adjoint!(b.nc)
    a = StepAdjoint(sizeof(StepAdjoint), ptr(lam.t_soisno), ptr(lam.h2osoi_liq), ptr(lam.h2osoi_ice),
                    ptr(lam.t_grnd), ptr(lam.t_h2osfc), ptr(lam.qcharge), ptr(grad.watsat), ptr(grad.bsw),
                    ptr(grad.sucsat), ptr(grad.hksat), ptr(lam.forc_lwrad))
    GC.@preserve ft_buf fw_buf begin
        check(ccall((:clmgb_column_step_vjp, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ptr{UInt8}, Ref{SwmConfig}, Float64, Int32,
                     Ptr{Cvoid}, Ptr{Cvoid}, Ref{StepAdjoint}, Ptr{UInt32}, Ptr{Cvoid}),
                    handle(), b, ft_buf, fw_buf, cfg, dtime, snow_method, ptr(t_ssbef), ptr(t_h2osfc_bef), a,
                    C_NULL, CUDA.stream().handle), "clmgb_column_step_vjp")
    end
    nothing
end

# Substep log (clmgb_substep_log): the forward step writes it, the reverse reads it,
# so the reverse runs neither the Richards substep loop nor soil_temperature! again.
# rec holds LOG_STRIDE(cap) Float64 per column, count one Int32 per column, st_rec
# LOG_ST_STRIDE Float64 per column (soil_temperature!'s factorisation and end state).
struct SubstepLog
    struct_size::Int64
    rec::Ptr{Cvoid}
    count::Ptr{Cvoid}
    cap::Int32
    st_rec::Ptr{Cvoid}
end
const LOG_REC = 25 + 2                  # CLMGB_MAX_NLEVSOI + 2
const LOG_FIN = 3 * 25 + 3
const LOG_ST_STRIDE = 464               # CLMGB_LOG_ST_STRIDE
log_stride(cap) = cap * LOG_REC + LOG_FIN
new_substep_log(nc::Integer, cap::Integer = 24) =
    (rec = CUDA.zeros(Float64, nc * log_stride(cap)), count = CUDA.fill(Int32(-1), nc), cap = Int32(cap),
     st_rec = CUDA.zeros(Float64, nc * LOG_ST_STRIDE))
log_struct(lg) = SubstepLog(sizeof(SubstepLog), ptr(lg.rec), ptr(lg.count), lg.cap, ptr(lg.st_rec))

function column_step_logged!(ft_buf, fw_buf, b::Bounds, cfg::SwmConfig, dtime, snow_method, t_ssbef,
                             t_h2osfc_bef, lg)
    GC.@preserve ft_buf fw_buf lg begin
        check(ccall((:clmgb_column_step_logged, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ptr{UInt8}, Ref{SwmConfig}, Float64, Int32,
                     Ptr{Cvoid}, Ptr{Cvoid}, Ref{SubstepLog}, Ptr{UInt32}, Ptr{Cvoid}),
                    handle(), b, ft_buf, fw_buf, cfg, dtime, snow_method, ptr(t_ssbef), ptr(t_h2osfc_bef),
                    log_struct(lg), C_NULL, CUDA.stream().handle), "clmgb_column_step_logged")
    end
    nothing
end

function column_step_vjp_logged!(ft_buf, fw_buf, b::Bounds, cfg::SwmConfig, dtime, snow_method, t_ssbef,
                                 t_h2osfc_bef, lam, grad, lg)
    TAPE_RESERVED[] || reserve_adjoint!(b.nc, 256)
    a = StepAdjoint(sizeof(StepAdjoint), ptr(lam.t_soisno), ptr(lam.h2osoi_liq), ptr(lam.h2osoi_ice),
                    ptr(lam.t_grnd), ptr(lam.t_h2osfc), ptr(lam.qcharge), ptr(grad.watsat), ptr(grad.bsw),
                    ptr(grad.sucsat), ptr(grad.hksat), ptr(lam.forc_lwrad))
    GC.@preserve ft_buf fw_buf lg begin
        check(ccall((:clmgb_column_step_vjp_logged, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ptr{UInt8}, Ref{SwmConfig}, Float64, Int32,
                     Ptr{Cvoid}, Ptr{Cvoid}, Ref{StepAdjoint}, Ref{SubstepLog}, Ptr{UInt32}, Ptr{Cvoid}),
                    handle(), b, ft_buf, fw_buf, cfg, dtime, snow_method, ptr(t_ssbef), ptr(t_h2osfc_bef), a,
                    log_struct(lg), C_NULL, CUDA.stream().handle), "clmgb_column_step_vjp_logged")
    end
    nothing
end

# The ChainRulesCore rrule and the Enzyme rules built on these calls are in
# CLMGB300ADExt.jl (a second extension, loaded with ChainRulesCore and Enzyme).

# ---------------------------------------------------------------------------
# Learned warm start: the first substep proposed by the perceptron (its weights are
# trained by the library's kernels: clmgb_mlp_*), then soil_water! from it.
# ---------------------------------------------------------------------------
function soil_water_warm!(fw_buf, b::Bounds, cfg::SwmConfig, dtime, dt_first::CuArray{Float64})
    GC.@preserve fw_buf begin
        check(ccall((:clmgb_soil_water_warm, lib), Int32,
                    (Ptr{Cvoid}, Ref{Bounds}, Ptr{UInt8}, Ref{SwmConfig}, Float64, Ptr{Cvoid}, Ptr{UInt32},
                     Ptr{Cvoid}),
                    handle(), b, fw_buf, cfg, dtime, ptr(dt_first), C_NULL, CUDA.stream().handle),
              "clmgb_soil_water_warm")
    end
    nothing
end

end # module
