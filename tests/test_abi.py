"""The C-ABI library loads, exports every entry point the header declares, and the
Python ctypes mirror matches the header's structs member by member (no GPU needed)."""
import ctypes as C
import os
import re

from clmgb import abi, _lib

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "clmgb.h")


def header_text():
    with open(HDR) as fh:
        return fh.read()


def declared_functions():
    txt = re.sub(r"/\*.*?\*/", "", header_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(clmgb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(_lib.exported_names()) == set(names)


def test_header_structs_match_ctypes():
    txt = header_text()
    for sname, fields in (("clmgb_soiltemp_fields", abi.SOILTEMP_FIELDS),
                          ("clmgb_soilwater_fields", abi.SOILWATER_FIELDS),
                          ("clmgb_rootsink_fields", abi.ROOTSINK_FIELDS),
                          ("clmgb_zd09_fields", abi.ZD09_FIELDS),
                          ("clmgb_soilflux_fields", abi.SOILFLUX_FIELDS),
                          ("clmgb_surfhyd_fields", abi.SURFHYD_FIELDS),
                          ("clmgb_snowlayer_fields", abi.SNOWLAYER_FIELDS),
                          ("clmgb_lake_fields", abi.LAKE_FIELDS),
                          ("clmgb_colbalance_fields", abi.COLBALANCE_FIELDS),
                          ("clmgb_flexcn_fields", abi.FLEXCN_FIELDS)):
        members = abi.header_struct_members(txt, sname)
        assert members[0] == "struct_size"
        assert members[1:] == [f[0] for f in fields], sname
    assert abi.header_struct_members(txt, "clmgb_varpar") == [f[0] for f in abi.Varpar._fields_]
    assert abi.header_struct_members(txt, "clmgb_bounds") == [f[0] for f in abi.Bounds._fields_]
    assert abi.header_struct_members(txt, "clmgb_swm_config") == [f[0] for f in abi.SwmConfig._fields_]
    assert abi.header_struct_members(txt, "clmgb_step_adjoint") == [f[0] for f in abi.StepAdjoint._fields_]
    assert abi.header_struct_members(txt, "clmgb_substep_log") == [f[0] for f in abi.SubstepLog._fields_]
    assert abi.header_struct_members(txt, "clmgb_surfhyd_config") == [f[0] for f in abi.SurfHydConfig._fields_]
    assert abi.header_struct_members(txt, "clmgb_snowlayer_config") == [f[0] for f in abi.SnowLayerConfig._fields_]
    assert abi.header_struct_members(txt, "clmgb_lake_config") == [f[0] for f in abi.LakeConfig._fields_]
    assert abi.header_struct_members(txt, "clmgb_balance_report") == [f[0] for f in abi.BalanceReport._fields_]


def test_header_constants_match_python():
    txt = header_text()
    consts = dict(re.findall(r"#define\s+CLMGB_(\w+)\s+(\d+)u?\b", txt))
    for name in ("COL_ADJ_UNSUPPORTED", "COL_TAPE_FULL", "OPT_ADJ_TAPE_USED", "OPT_ADJ_TAPE_SLOTS",
                 "OPT_ADJ_TAPE_ENTRIES", "OPT_STEP_SCHEDULE", "OPT_WAVES_OCCUPANCY", "OPT_ADJ_RICHARDS",
                 "ADJ_RICHARDS_CLOSED_FORM", "ADJ_RICHARDS_RECORDED", "COL_ADJ_REPLAY", "ADJ_MAX_SUBSTEPS",
                 "OPT_ADJ_SOIL_TEMPERATURE", "ADJ_ST_CLOSED_FORM", "ADJ_ST_RECORDED", "OPT_QUEUE_FRESH_BATCH", "OPT_COLUMN_BASE", "OPT_QUEUE_DEFER",
                 "COL_FILTER", "OPT_ATTEMPT_CAP", "OPT_QUEUE_POLL_LIMIT", "OPT_QUEUE_PUBLISH_DELAY",
                 "OPT_COUNT_WORK", "OPT_WORK_LEVEL_ATTEMPTS", "OPT_WORK_LEVEL_REFRESHES", "COL_QUEUE_WAIT",
                 "LOG_ST_STRIDE", "OPT_RECORDS_TMA", "OPT_RECORDS_TMA_USED", "COL_COPY_WAIT",
                 "OPT_TRIDIAG_METHOD", "TRIDIAG_THOMAS", "TRIDIAG_PCR", "OPT_ST_BLOCK"):
        assert int(consts[name]) == getattr(abi, name), name
    for name in ("SH_FLOODC", "SH_SAT_EXCESS", "SH_QFLX_INPUTS", "SH_INFL_EXCESS", "SH_ROUTE", "SH_UPDATE_H2OSFC",
                 "SH_INFILTRATION", "SH_TOTAL_RUNOFF", "SH_URBAN_PONDING", "SH_ALL", "FSAT_TOPMODEL", "FSAT_VIC",
                 "QINMAX_NONE", "QINMAX_HKSAT", "SL_COMPACTION", "SL_COMBINE", "SL_DIVIDE", "SL_ZERO_EMPTY",
                 "SL_FILTER", "SL_ALL", "OVERBURDEN_ANDERSON1976", "OVERBURDEN_VIONNET2012"):
        assert int(consts[name]) == getattr(abi, name), name


def test_abi_version_and_errors():
    lib = _lib.load()
    assert lib.clmgb_abi_version() == 1
    assert b"sm_103a" in lib.clmgb_build_info()
    assert lib.clmgb_strerror(abi.CLMGB_ERR_CONFIG)
    # host-side argument checks run before any CUDA call
    h = C.c_void_p()
    assert lib.clmgb_create(None, C.byref(h)) == abi.CLMGB_ERR_NULL_ARG
    bad = abi.Varpar(13, 25, 20, 5, 25, 0)
    assert lib.clmgb_create(C.byref(bad), C.byref(h)) == abi.CLMGB_ERR_DIMS
    bad = abi.Varpar(12, 25, 20, 5, 24, 0)
    assert lib.clmgb_create(C.byref(bad), C.byref(h)) == abi.CLMGB_ERR_DIMS
    assert lib.clmgb_soil_temperature(None, None, None, 1800.0, 1, 0, None, None) == abi.CLMGB_ERR_HANDLE


def test_product_package_never_imports_oracle():
    """The product path must not load the oracle (no CPU fallback)."""
    pkg = os.path.join(os.path.dirname(HDR), "..", "clm.jl_gb300")
    pat = re.compile(r"(import\s+oracle|from\s+oracle|clmoracle|\borc_)")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".jl")):
                with open(os.path.join(root, f)) as fh:
                    assert not pat.search(fh.read()), f
