"""The reference's model switches at the boundary (wg_model_options): every
value outside the built set is refused by wg_create with WG_ERR_UNSUPPORTED and
the option's name, before any device is touched, so a caller running the
reference with another option never gets a silently different model (runs on
the CPU: the refusal comes before the device check)."""
import numpy as np
import pytest

from watergap2_gb300 import synthetic as sy

# option -> a value of the reference's option file that is not built
REFUSED = {
    "time_series": 0, "cloud": 0, "intercept": 0, "calc_albedo": 1, "use_kc": 1, "pet_opt": 1,
    "clcl_opt": 1, "perma_opt": 1, "glacier_opt": 1, "land_cover_opt": 1, "arid_area_opt": 1,
    "river_evapo_opt": 1, "statcorr_opt": 2, "use_alloc": 1, "aggr_nus_glo_lak_res_opt": 2,
    "ant_nat_opt": 1, "res_year_opt": 1, "climate_spatial_resolution": 1,
}
NAMES = {"pet_opt": "petOpt", "clcl_opt": "clclOpt", "perma_opt": "permaOpt", "glacier_opt": "glacierOpt",
         "land_cover_opt": "landCoverOpt", "arid_area_opt": "aridareaOpt", "river_evapo_opt": "riverEvapoOpt",
         "statcorr_opt": "statcorrOpt", "aggr_nus_glo_lak_res_opt": "aggrNUsGloLakResOpt",
         "ant_nat_opt": "antNatOpt", "res_year_opt": "resYearOpt"}


@pytest.fixture(scope="module")
def region():
    from watergap2_gb300 import build, gpu
    import os
    if not os.path.exists(gpu.LIB_PATH):
        build.build()
    return sy.region_small_swb(seed=3)


@pytest.mark.parametrize("option", sorted(REFUSED))
def test_unbuilt_option_is_refused(region, option):
    from watergap2_gb300.gpu import Model, WgError
    with pytest.raises(WgError, match=rf"unsupported.*options\.{NAMES.get(option, option)} = "):
        Model(region, max_days=2, model_options={option: REFUSED[option]})


def test_defaults_match_the_reference_configuration():
    import ctypes
    from watergap2_gb300 import gpu
    lib = gpu.load_library()
    m = gpu._ModelOptions()
    lib.wg_model_options_default(ctypes.byref(m))
    got = {f: getattr(m, f) for f in gpu.MODEL_OPTIONS}
    want = dict.fromkeys(gpu.MODEL_OPTIONS, 0)
    want.update(time_series=1, cloud=2, intercept=1, res_opt=1)
    assert got == want


def test_built_values_pass_the_option_check(region):
    """Built values get past the option check (on a host without a GPU wg_create
    then stops at the device check)."""
    from watergap2_gb300.gpu import Model, WgError
    for opts, reg in (({}, region), ({"statcorr_opt": 1}, region),
                      ({"res_opt": 0}, sy.region_64x64(size=8))):   # resOpt 0: a region without reservoirs
        try:
            Model(reg, max_days=2, model_options=opts)
        except WgError as exc:
            assert "unsupported" not in str(exc), (opts, exc)


def test_res_opt_zero_refused_with_reservoirs(region):
    from watergap2_gb300.gpu import Model, WgError
    assert np.any(region.res_area > 0)
    with pytest.raises(WgError, match=r"options\.resOpt = 0"):
        Model(region, max_days=2, model_options={"res_opt": 0})


def test_station_correction_with_water_temperature_refused(region):
    from watergap2_gb300.gpu import Model, WgError
    with pytest.raises(WgError, match="statcorrOpt = 1 together with calc_wtemp"):
        Model(region.with_options(statcorr_opt=1), max_days=2, water_temp=True)


def test_glwd_aggregation_conditions(region):
    """aggrNUsGloLakResOpt = 1 (Model(glwd_unit=...)) needs water use and the
    units, and is built for FP64, one member, without the water temperature;
    units where an outflow cell has none, or a unit has two outflow cells, are
    refused with the reason; a valid set gets past the checks (on a host without
    a GPU wg_create then stops at the device check)."""
    from watergap2_gb300.gpu import Model, WgError
    unit = sy.glwd_units(region)
    with pytest.raises(WgError, match="needs water use"):
        Model(region, max_days=2, glwd_unit=unit)
    with pytest.raises(WgError, match="unsupported.*FP64, one member"):
        Model(region, max_days=2, water_use=True, glwd_unit=unit, precision="fp32")
    with pytest.raises(WgError, match="unsupported.*FP64, one member"):
        Model(region, max_days=2, water_use=True, glwd_unit=unit, water_temp=True)
    outflow = np.nonzero((region.lake_area > 0) | (region.res_area > 0))[0]
    bad = unit.copy()
    bad[outflow[0]] = 0
    with pytest.raises(WgError, match="has no unit"):
        Model(region, max_days=2, water_use=True, glwd_unit=bad)
    bad = unit.copy()
    bad[outflow[1]] = bad[outflow[0]]
    with pytest.raises(WgError, match="2 outflow cells"):
        Model(region, max_days=2, water_use=True, glwd_unit=bad)
    for wu in (1, 2):
        try:
            Model(region, max_days=2, water_use=wu, glwd_unit=unit)
        except WgError as exc:
            assert "invalid" not in str(exc) and "unsupported" not in str(exc), exc
