"""A Wflow TOML configuration driving the file helpers (wflow_gb300.config) on the CPU.

The TOML here follows the reference's schema (Wflow/src/config_structure.jl): domain maps under
[input], parameters under [input.static] in the three entry forms (a variable name, a constant
{value = v}, {netcdf_variable_name, scale, offset}), forcing under [input.forcing], states under
[state.variables], paths relative to the TOML's folder and dir_input / dir_output. A model set
up from it runs like the model built from the arrays the files were written from.
"""


import numpy as np
import pytest

from wflow_gb300 import abi, forcing, staticmaps, states, synthetic
from wflow_gb300.config import WflowConfig
import oracle_py as O

F = abi.FIELD
FILE_NAMES = {"basin__local_drain_direction": "wflow_ldd", "river_location__mask": "wflow_river",
              "subbasin_location__count": "wflow_subcatch", "soil__thickness": "SoilThickness",
              "soil_water__saturated_volume_fraction": "thetaS", "land_surface__slope": "Slope",
              "soil_surface_water__vertical_saturated_hydraulic_conductivity": "KsatVer"}

TOML = """
dir_input = "data/input"
dir_output = "data/output"

[time]
calendar = "proleptic_gregorian"
starttime = 2000-01-01T00:00:00
endtime = 2000-01-05T00:00:00
time_units = "days since 1900-01-01 00:00:00"
timestepsecs = 86400

[state]
path_input = "instates.nc"
path_output = "outstates.nc"

[state.variables]
vegetation_canopy_water__depth = "canopystorage"
soil_water_saturated_zone__depth = "satwaterdepth"
soil_surface__temperature = "tsoil"
soil_layer_water_unsaturated_zone__depth = "ustorelayerdepth"
snowpack_dry_snow__leq_depth = "snow"
snowpack_liquid_water__depth = "snowwater"
river_water__depth = "h_river"
river_water__instantaneous_volume_flow_rate = "q_river"
subsurface_water__instantaneous_volume_flow_rate = "ssf"
land_surface_water__instantaneous_volume_flow_rate = "q_land"
land_surface_water__depth = "h_land"

[input]
path_forcing = "forcing.nc"
path_static = "staticmaps.nc"
basin__local_drain_direction = "wflow_ldd"
river_location__mask = "wflow_river"
subbasin_location__count = "wflow_subcatch"

[input.forcing]
atmosphere_water__precipitation_volume_flux = "precip"
land_surface_water__potential_evaporation_volume_flux = "pet"
atmosphere_air__temperature = "temp"

[input.static]
soil__thickness = "SoilThickness"
soil_water__saturated_volume_fraction = "thetaS"
land_surface__slope = "Slope"
vegetation__crop_factor = { value = 1.0 }

[input.static.soil_surface_water__vertical_saturated_hydraulic_conductivity]
netcdf_variable_name = "KsatVer"
scale = 1.0
offset = 0.0

[model]
type = "sbm"
snow__flag = true
cold_start__flag = true
water_mass_balance__flag = true
kinematic_wave__adaptive_time_step_flag = false
soil_layer__thickness = [100, 300, 800]
"""


@pytest.fixture()
def setup(tmp_path):
    (tmp_path / "data" / "input").mkdir(parents=True)
    (tmp_path / "data" / "output").mkdir(parents=True)
    (tmp_path / "sbm.toml").write_text(TOML)
    dom = synthetic.make_domain(16, 1000.0, seed=3)
    dom.params["crop_coefficient"] = np.ones(dom.n_land)
    staticmaps.write_staticmaps(dom, tmp_path / "data" / "input" / "staticmaps.nc", names=FILE_NAMES)
    return tmp_path, dom


def test_settings_and_paths(setup):
    root, _ = setup
    cfg = WflowConfig(root / "sbm.toml")
    assert cfg.path_static == root / "data" / "input" / "staticmaps.nc"
    assert cfg.state_output == root / "data" / "output" / "outstates.nc"
    assert cfg.static["basin__local_drain_direction"] == {"name": "wflow_ldd"}
    assert cfg.static["vegetation__crop_factor"] == {"value": 1.0}
    assert cfg.static["soil_surface_water__vertical_saturated_hydraulic_conductivity"] == {
        "name": "KsatVer", "scale": 1.0, "offset": 0.0}
    c = cfg.wf_config()
    assert c.dt == 86400.0 and c.snow == 1 and c.water_mass_balance == 1 and c.n_soil_layer_thickness == 3
    assert [t.day for t in cfg.times()] == [2, 3, 4, 5]


def test_unsupported_options_are_refused(setup):
    root, _ = setup
    text = TOML.replace('type = "sbm"', 'type = "sbm"\ndrain__flag = true\nland_routing = "local_inertial"')
    (root / "g.toml").write_text(text)
    with pytest.raises(ValueError, match="drain__flag.*land_routing"):
        WflowConfig(root / "g.toml").wf_config()


def test_snow_transport_and_glacier_flags(setup):
    root, _ = setup
    text = TOML.replace('type = "sbm"', 'type = "sbm"\nglacier__flag = true\nsnow_gravitational_transport__flag = true')
    (root / "sg.toml").write_text(text)
    c = WflowConfig(root / "sg.toml").wf_config()
    assert c.snow == 1 and c.glacier == 1 and c.snow_gravitational_transport == 1
    # a glacier needs the snow model (sbm.jl:45-49); the transport without snow does nothing
    (root / "ns.toml").write_text(text.replace("snow__flag = true", "snow__flag = false"))
    with pytest.raises(ValueError, match="glacier__flag without snow"):
        WflowConfig(root / "ns.toml").wf_config()


def test_model_from_the_toml_runs_like_the_arrays(setup):
    root, dom = setup
    cfg = WflowConfig(root / "sbm.toml")
    got, grid, _ = staticmaps.load_staticmaps(cfg.path_static, mapping=cfg.static)
    for k, v in dom.params.items():
        if v is not None:
            np.testing.assert_allclose(got.params[k], v, rtol=4e-16, atol=0, err_msg=k)
    times = cfg.times()
    arrs = [synthetic.forcing(s, cfg.dt, dom.n_land, seed=1) for s in range(len(times))]
    forcing.write_forcing(cfg.path_forcing, grid, times, [a[0] for a in arrs], [a[1] for a in arrs],
                          [a[2] for a in arrs], cfg.dt, time_units=cfg.time_units)
    ff = forcing.ForcingFile(cfg.path_forcing, grid, cfg.dt, mapping=cfg.forcing)
    wcfg = cfg.wf_config()
    a, b = O.OracleModel(wcfg, dom), O.OracleModel(wcfg, got)
    for k, t in enumerate(times):
        a.set_forcing(*arrs[k])
        a.step()
        b.set_forcing(*ff.at(t))
        b.step()
    for f in ("RIVER_Q", "SATURATED_WATER_DEPTH", "SNOW_STORAGE", "SSF_Q"):
        x, y = a.get(F[f]), b.get(F[f])
        assert np.max(np.abs(x - y) / np.maximum(np.abs(x), 1e-300)) <= 1e-12, f
    # the end state under the TOML's variable names, and a warm start from it
    states.write_states(b, got, cfg.state_output, grid=grid, ncnames=cfg.state_ncnames, time=4.0)
    from wflow_gb300 import ncio
    names = set(ncio.NcFile(cfg.state_output).variables)
    assert {"satwaterdepth", "ustorelayerdepth", "q_river", "ssf", "h_land"} <= names
    c = O.OracleModel(wcfg, got)
    states.read_states(c, got, cfg.state_output, grid=grid, ncnames=cfg.state_ncnames)
    x, y = b.get(F["SATURATED_WATER_DEPTH"]), c.get(F["SATURATED_WATER_DEPTH"])
    assert np.max(np.abs(x - y) / x) <= 1e-15


def test_scale_and_offset_entries(setup):
    root, dom = setup
    path = root / "data" / "input" / "staticmaps.nc"
    base, _, _ = staticmaps.load_staticmaps(path, mapping={**{k: v for k, v in FILE_NAMES.items()}})
    m = dict(FILE_NAMES)
    m["soil__thickness"] = {"netcdf_variable_name": "SoilThickness", "scale": 0.5, "offset": 100.0}
    got, _, _ = staticmaps.load_staticmaps(path, mapping=m)
    # file value (mm) * 0.5 + 100 mm, then to metres
    expect = ((base.params["soil_thickness"] / 1e-3) * 0.5 + 100.0) * 1e-3
    np.testing.assert_allclose(got.params["soil_thickness"], expect, rtol=1e-15)


# ---- the reference's own test configurations (tests/golden/reference_configs.json, copied from
# Wflow/test by tests/golden/make_reference_configs.py)
def _reference_config(tmp_path, name):
    import json
    from pathlib import Path
    data = json.loads((Path(__file__).parent / "golden" / "reference_configs.json").read_text())
    p = tmp_path / name
    p.write_text(data[name]["text"])
    return WflowConfig(p)


def test_reference_sbm_config_parses(tmp_path):
    cfg = _reference_config(tmp_path, "sbm_config.toml")
    root = tmp_path
    assert cfg.dt == 86400.0
    assert (cfg.starttime.year, cfg.starttime.month, cfg.starttime.day) == (2000, 1, 1)
    assert (cfg.endtime.year, cfg.endtime.month, cfg.endtime.day) == (2000, 2, 1)
    assert len(cfg.times()) == 31
    assert cfg.path_static == root / "data" / "input" / "staticmaps-moselle.nc"
    assert cfg.path_forcing == root / "data" / "input" / "forcing-moselle.nc"
    assert cfg.state_input == root / "data" / "input" / "instates-moselle.nc"
    assert cfg.state_output == root / "data" / "output" / "outstates-moselle.nc"
    assert cfg.static["basin__local_drain_direction"] == {"name": "wflow_ldd"}
    assert cfg.static["soil_surface_water__vertical_saturated_hydraulic_conductivity"] == {
        "name": "KsatVer", "scale": 1.0, "offset": 0.0}
    assert cfg.forcing["atmosphere_water__precipitation_volume_flux"] == {"name": "precip"}
    assert cfg.state_ncnames["soil_water_saturated_zone__depth"] == "satwaterdepth"
    assert cfg.reservoirs and cfg.cold_start
    # outside the GPU step: leaf-area-index driven interception, and snow transport with reservoirs
    with pytest.raises(ValueError) as e:
        cfg.wf_config()
    assert "cyclic LAI" in str(e.value) and "snow_gravitational_transport__flag with reservoir__flag" in str(e.value)


def test_reference_sbm_simple_parses(tmp_path):
    cfg = _reference_config(tmp_path, "sbm_simple.toml")
    assert cfg.dt == 86400.0  # the reference's default time step
    assert (cfg.endtime.year, cfg.endtime.month, cfg.endtime.day) == (2000, 1, 10)
    assert cfg.static["soil__thickness"] == {"name": "SoilThickness"}
    assert not cfg.reservoirs
    with pytest.raises(ValueError, match="cyclic LAI"):
        cfg.wf_config()
    # without the cyclic LAI the rest of the [model] section maps onto the step's configuration
    cfg.raw["input"].pop("cyclic")
    c = cfg.wf_config()
    assert c.n_soil_layer_thickness == 3 and c.snow == 0 and c.glacier == 0
    assert abs(c.soil_layer_thickness[2] - 0.8) < 1e-15
