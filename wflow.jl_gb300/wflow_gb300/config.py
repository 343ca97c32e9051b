"""A Wflow TOML configuration read for the files and settings the GPU step needs.

Follows the reference's configuration schema (Wflow/src/config_structure.jl, config_init.jl):
  [time]             starttime, endtime, timestepsecs, calendar, time_units
  [model]            the flags of the SBM path (snow, gravitational snow transport, glacier,
                     reservoirs, adaptive kinematic-wave sub-steps, sub-step sizes, soil layers, Kv
                     profile, mass balance, ...)
  [input]            path_static, path_forcing and the domain maps (LDD, river, subbasin, ...)
  [input.static]     standard name -> netCDF variable (Option 3: a name), a constant
                     ({value = v}, Option 2) or {netcdf_variable_name, scale, offset, layer}
                     (Option 1; config_init.jl:113-156, applied as apply_affine_transform!,
                     utils.jl:239-256)
  [input.forcing]    the forcing variables, in the same forms
  [state]            path_input, path_output and [state.variables] (standard name -> name)
Relative paths are relative to the TOML's folder and dir_input / dir_output, as in Wflow
(config_utils.jl input_path / output_path).
"""

import datetime as _dt
from pathlib import Path

from . import abi

try:
    import tomllib as _toml
except ImportError:  # Python < 3.11
    _toml = None

# options of the reference that this step does not run (the caller keeps Wflow's own update)
UNSUPPORTED_FLAGS = ("floodplain_1d__flag", "drain__flag", "constanthead__flag", "pit__flag")


def _entry(v):
    """Normalise an [input] entry to {"name", "scale", "offset", "layer"} or {"value"}."""
    if isinstance(v, str):
        return {"name": v}
    if isinstance(v, (int, float)):
        return {"value": float(v)}
    if isinstance(v, dict):
        if "netcdf_variable_name" in v or "name" in v:  # the TOML form, or an already normalised entry
            e = {"name": v.get("netcdf_variable_name", v.get("name"))}
            for k in ("scale", "offset", "layer"):
                if k in v:
                    e[k] = v[k]
            return e
        if "value" in v:
            return {"value": v["value"]}
    raise ValueError(f"cannot parse the [input] entry {v!r}")


class WflowConfig:
    """The parts of a Wflow TOML the GPU step uses."""

    def __init__(self, path):
        if _toml is None:
            raise RuntimeError("reading TOML needs Python 3.11 or later (tomllib)")
        self.path = Path(path)
        with open(self.path, "rb") as fh:
            self.raw = _toml.load(fh)
        root = self.path.parent
        self.dir_input = root / self.raw.get("dir_input", ".")
        self.dir_output = root / self.raw.get("dir_output", ".")
        t = self.raw.get("time", {})
        self.dt = float(t.get("timestepsecs", 86400))
        self.starttime = _as_datetime(t.get("starttime"))
        self.endtime = _as_datetime(t.get("endtime"))
        self.calendar = t.get("calendar", "standard")
        self.time_units = t.get("time_units", "days since 1900-01-01 00:00:00")
        self.model = dict(self.raw.get("model", {}))
        inp = self.raw.get("input", {})
        self.path_static = self.dir_input / inp["path_static"] if "path_static" in inp else None
        self.path_forcing = self.dir_input / inp["path_forcing"] if "path_forcing" in inp else None
        static = {}
        for k, v in inp.items():  # domain maps given directly under [input]
            if k in ("path_static", "path_forcing", "static", "forcing", "cyclic") or k.startswith("path_"):
                continue
            if isinstance(v, (str, dict)):
                static[k] = _entry(v)
        for k, v in inp.get("static", {}).items():
            static[k] = _entry(v)
        self.static = static
        self.forcing = {k: _entry(v) for k, v in inp.get("forcing", {}).items()}
        st = self.raw.get("state", {})
        self.state_input = self.dir_input / st["path_input"] if "path_input" in st else None
        self.state_output = self.dir_output / st["path_output"] if "path_output" in st else None
        self.state_ncnames = dict(st.get("variables", {}))

    @property
    def reservoirs(self):
        return bool(self.model.get("reservoir__flag", False))

    @property
    def cold_start(self):
        return bool(self.model.get("cold_start__flag", True))

    def check_supported(self):
        """Raise for options outside the GPU step (the Julia shim's check_supported)."""
        bad = [f for f in UNSUPPORTED_FLAGS if self.model.get(f, False)]
        if self.model.get("type", "sbm") != "sbm":
            bad.append(f"model type {self.model.get('type')}")
        for k in ("land_routing", "river_routing"):
            if self.model.get(k, "kinematic_wave") != "kinematic_wave":
                bad.append(f"{k} {self.model[k]}")
        if "water_demand" in self.model:
            bad.append("water demand")
        prof = self.model.get("saturated_hydraulic_conductivity_profile", "exponential")
        if prof not in ("exponential", "exponential_constant"):
            bad.append(f"saturated_hydraulic_conductivity_profile {prof}")
        if "vegetation__leaf_area_index" in self.raw.get("input", {}).get("cyclic", {}):
            bad.append("leaf-area-index driven interception (cyclic LAI)")
        snow = self.model.get("snow__flag", False)
        if self.model.get("glacier__flag", False) and not snow:
            bad.append("glacier__flag without snow__flag (the reference refuses it, sbm.jl:45-49)")
        if snow and self.model.get("snow_gravitational_transport__flag", False) and self.reservoirs:
            bad.append("snow_gravitational_transport__flag with reservoir__flag")
        if bad:
            raise ValueError("not supported by the GPU step: " + ", ".join(bad))

    def wf_config(self, form=abi.WF_FORM_FP64, n_members=1):
        """The WfConfig of the [model] and [time] sections."""
        self.check_supported()
        m = self.model
        c = abi.WfConfig()
        c.dt = self.dt
        layers = [float(x) for x in m.get("soil_layer__thickness", [100, 300, 800])]
        if len(layers) + 1 > abi.WF_MAX_LAYERS:
            raise ValueError("more soil layers than the GPU step holds")
        c.n_soil_layer_thickness = len(layers)
        for i, t in enumerate(layers):
            c.soil_layer_thickness[i] = t * 1e-3
        c.snow = int(bool(m.get("snow__flag", False)))
        # without snow the transport is a no-op in the reference (surface_process.jl:21)
        c.snow_gravitational_transport = int(c.snow and bool(m.get("snow_gravitational_transport__flag", False)))
        c.glacier = int(bool(m.get("glacier__flag", False)))
        c.soil_infiltration_reduction = int(bool(m.get("soil_infiltration_reduction__flag", False)))
        c.water_mass_balance = int(bool(m.get("water_mass_balance__flag", False)))
        c.adaptive_timestep = int(bool(m.get("kinematic_wave__adaptive_time_step_flag", False)))
        prof = m.get("saturated_hydraulic_conductivity_profile", "exponential")
        c.kv_profile = abi.WF_KV_EXPONENTIAL if prof == "exponential" else abi.WF_KV_EXPONENTIAL_CONSTANT
        c.land_dt_fixed = float(m.get("land_kinematic_wave__time_step", 3600.0))
        c.river_dt_fixed = float(m.get("river_kinematic_wave__time_step", 900.0))
        c.subsurface_dt_fixed = float(m.get("subsurface_kinematic_wave__time_step", 86400.0))
        c.subsurface_alpha = float(m.get("subsurface_kinematic_wave__alpha_coefficient", 1.0))
        c.form = int(form)
        c.n_members = int(n_members)
        c.per_member_soil = 0
        return c

    def times(self):
        """Model times of the steps (the clock after each advance!, Wflow.jl:311-322)."""
        out = []
        t = self.starttime
        step = _dt.timedelta(seconds=self.dt)
        while t + step <= self.endtime:
            t = t + step
            out.append(t)
        return out


def julian_day(t):
    """Day of the year with leap days not counted (Wflow's julian_day, utils.jl:674-678):
    February 28 is day 59 and March 1 day 60 in every year."""
    doy = t.timetuple().tm_yday
    leap = t.year % 4 == 0 and (t.year % 100 != 0 or t.year % 400 == 0)
    return doy - (1 if leap and doy > 60 else 0)


def rating_curve_day(time, dt):
    """The H-Q tables' column of the step that ends at `time` (update_index_hq!,
    routing/surface/reservoir.jl:379-385: julian_day(clock.time - clock.dt))."""
    return julian_day(time - _dt.timedelta(seconds=float(dt)))


def _as_datetime(v):
    if v is None:
        return None
    if isinstance(v, _dt.datetime):
        return v
    if isinstance(v, _dt.date):
        return _dt.datetime(v.year, v.month, v.day)
    return _dt.datetime.fromisoformat(str(v))
