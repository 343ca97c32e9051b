"""Extract the known-answer tests (KATs) of Wflow.jl's unit tests into reference_kats.json.

Wflow.jl's unit tests (Wflow/test/land_process.jl, soil.jl, routing_process.jl, reservoir.jl,
utils.jl)
hold input/output literals for every process function on the SBM + kinematic-wave path.
Julia is not available to run them, so this script reads the test files as text and
copies each literal from the cited line. Each case records the function, its inputs, the
expected outputs, the comparison Julia uses (`==` or `≈`, i.e. rtol = sqrt(eps)), and the
file:line every number came from.

Usage: python tests/golden/make_reference_kats.py <path-to-Wflow.jl-checkout>
(or with the checkout path in the environment variable WFLOW_JL_CHECKOUT).
"""

import json
import re
import sys
from pathlib import Path


def _checkout():
    import os
    p = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WFLOW_JL_CHECKOUT")
    if not p:
        sys.exit("usage: make_reference_kats.py <path-to-Wflow.jl-checkout> (or set WFLOW_JL_CHECKOUT)")
    return Path(p)


REF = _checkout() / "Wflow" / "test"
OUT = Path(__file__).with_name("reference_kats.json")

_lines_cache = {}


def _lines(fname):
    if fname not in _lines_cache:
        _lines_cache[fname] = (REF / fname).read_text().splitlines()
    return _lines_cache[fname]


_TOK = re.compile(r"[A-Za-z_][A-Za-z_0-9]*|-?\d+(?:\.\d*)?(?:[eE][-+]?\d+)?")


def nums(fname, line, count=None):
    """Numeric literals (NaN included) on a (1-based) line of a reference test file (Julia's
    digit separators, as in 25_000_000.0, are dropped first)."""
    vals = []
    for tok in _TOK.findall(re.sub(r"(?<=\d)_(?=\d)", "", _lines(fname)[line - 1])):
        if tok == "NaN":
            vals.append(float("nan"))
        elif tok[0].isdigit() or tok[0] == "-":
            vals.append(float(tok))
    return vals if count is None else vals[:count]


def num(fname, line, k=-1):
    """k-th numeric literal on a (1-based) line of a reference test file (default: the last,
    which skips index literals such as `x[1]` in `@test x[1] ≈ value`)."""
    return nums(fname, line)[k]


def span(fname, first, last):
    vals = []
    for ln in range(first, last + 1):
        vals += nums(fname, ln)
    return vals


def case(cid, fn, src, args, expect, cmp="approx", note=None, prev=None):
    d = {"id": cid, "fn": fn, "src": src, "args": args, "expect": expect, "cmp": cmp}
    if prev:
        d["prev"] = prev
    if note:
        d["note"] = note
    return d


def build():
    L, S, R, U = "land_process.jl", "soil.jl", "routing_process.jl", "utils.jl"
    K = []
    # ---------------------------------------------------------------- land_process.jl
    dt = num(L, 3)
    gash = dict(dt=dt, maximum_canopy_storage=num(L, 6), evaporation_to_precipitation_ratio=num(L, 7),
                canopy_gap_fraction=num(L, 8), precipitation=num(L, 9), canopy_storage=num(L, 10),
                max_evaporation=num(L, 11))
    K.append(case("gash_no_canopy", "rainfall_interception_gash", f"{L}:1-25", dict(gash),
                  dict(throughfall=gash["precipitation"], interception=0.0, stem_flow=0.0,
                       canopy_storage=gash["canopy_storage"]), cmp="exact"))
    g2 = dict(gash, maximum_canopy_storage=num(L, 28))
    K.append(case("gash_large_storm", "rainfall_interception_gash", f"{L}:27-42", g2,
                  dict(throughfall=num(L, 39), interception=num(L, 40), stem_flow=num(L, 41),
                       canopy_storage=gash["canopy_storage"])))
    g3 = dict(g2, precipitation=num(L, 45))
    K.append(case("gash_small_storm", "rainfall_interception_gash", f"{L}:44-59", g3,
                  dict(throughfall=num(L, 56), interception=num(L, 57), stem_flow=num(L, 58),
                       canopy_storage=gash["canopy_storage"])))
    mr = dict(dt=num(L, 63), precipitation=num(L, 66), potential_evaporation=num(L, 67),
              canopy_storage=num(L, 68), canopy_gap_fraction=num(L, 69), maximum_canopy_storage=num(L, 70))
    K.append(case("modrut_gap_small", "rainfall_interception_modrut", f"{L}:62-82", dict(mr),
                  dict(throughfall=num(L, 79), canopy_evap=num(L, 80), stemflow=num(L, 81),
                       canopy_storage=num(L, 82))))
    # second modrut call reuses canopy_storage returned by the first call
    mr2 = dict(mr, precipitation=num(L, 85), canopy_gap_fraction=num(L, 86), canopy_storage="$prev.canopy_storage")
    K.append(case("modrut_gap_large", "rainfall_interception_modrut", f"{L}:84-98", mr2,
                  dict(throughfall=num(L, 95), canopy_evap=num(L, 96), stemflow=num(L, 97),
                       canopy_storage=num(L, 98)),
                  note="canopy_storage input is the output of the previous call (line 71)",
                  prev="modrut_gap_small"))
    ph = dict(precipitation=num(L, 105), temperature=num(L, 106), temperature_interval_snowfall=num(L, 107),
              temperature_threshold_snowfall=num(L, 108))
    K.append(case("precip_hbv_interval", "precipitation_hbv", f"{L}:104-116", dict(ph),
                  dict(snow_precip=num(L, 115), liquid_precip=num(L, 116))))
    K.append(case("precip_hbv_warm", "precipitation_hbv", f"{L}:118-128",
                  dict(ph, temperature_interval_snowfall=num(L, 120)),
                  dict(snow_precip=0.0, liquid_precip=ph["precipitation"]), cmp="exact"))
    K.append(case("precip_hbv_cold", "precipitation_hbv", f"{L}:130-139",
                  dict(ph, temperature_interval_snowfall=num(L, 120), temperature=num(L, 131)),
                  dict(snow_precip=ph["precipitation"], liquid_precip=0.0), cmp="exact"))
    sp = dict(dt=num(L, 143), snow_storage=num(L, 145), snow_water=num(L, 146), snow_precip=num(L, 147),
              liquid_precip=num(L, 148), temperature=num(L, 149), temperature_threshold_melt=num(L, 150),
              degree_day_factor=num(L, 151), water_holding_capacity=num(L, 152))
    K.append(case("snowpack_melt", "snowpack_hbv", f"{L}:142-170", dict(sp),
                  dict(snow_storage=num(L, 166), snow_water=num(L, 167), snow_water_equivalent=num(L, 168),
                       snow_melt=num(L, 169), runoff=num(L, 170))))
    K.append(case("snowpack_refreeze", "snowpack_hbv", f"{L}:172-190",
                  dict(sp, temperature=num(L, 173), snow_water="$prev.snow_water"),
                  dict(snow_storage=num(L, 186), snow_water=num(L, 187), snow_water_equivalent=num(L, 188),
                       snow_melt=num(L, 189), runoff=num(L, 190)),
                  note="snow_water input is the output of the previous call (line 154 rebinds it)",
                  prev="snowpack_melt"))
    gl = dict(dt=num(L, 194), glacier_fraction=num(L, 196), glacier_store=num(L, 197), snow_storage=num(L, 198),
              temperature=num(L, 199), temperature_threshold_melt=num(L, 200), degree_day_factor=num(L, 201),
              snow_to_ice_fraction=num(L, 202), maximum_snow_to_ice_rate=num(L, 203))
    K.append(case("glacier_hbv", "glacier_hbv", f"{L}:193-219", gl,
                  dict(snow_storage=num(L, 215), snow_to_glacier=num(L, 216), glacier_storage=num(L, 217),
                       glacier_melt=num(L, 218))))
    inf = dict(dt=num(L, 222), potential_infiltration=num(L, 224), compacted_soil_area_fraction=num(L, 225),
               infiltration_capacity_soil=num(L, 226), infiltration_capacity_compacted_soil=num(L, 227),
               unsaturated_store_capacity=num(L, 228), f_infiltration_reduction=num(L, 229))
    K.append(case("infiltration", "infiltration", f"{L}:221-241", inf, dict(infiltration_excess=num(L, 240))))
    uz = dict(dt=num(L, 244), kv_z=num(L, 246), l_sat=num(L, 247), c=num(L, 248))
    K.append(case("unsatzone_flow_layer_wet", "unsatzone_flow_layer", f"{L}:250-254",
                  dict(uz, usd=num(L, 251)), dict(usd=num(L, 253), sum_ast_times_dt=num(L, 254)),
                  note="the reference assigns these outputs but never asserts them; the assigned "
                       "`sum_ast` equals the returned rate times dt (a value in metres)"))
    K.append(case("unsatzone_flow_layer_dry", "unsatzone_flow_layer", f"{L}:256-260",
                  dict(uz, usd=num(L, 257)), dict(usd=0.0, sum_ast=0.0), cmp="exact"))
    bc = dict(volumetric_water_content=num(L, 266), theta_s=num(L, 267), theta_r=num(L, 268), c=num(L, 269),
              air_entry_pressure=num(L, 270))
    K.append(case("head_brooks_corey", "head_brooks_corey", f"{L}:265-280", dict(bc),
                  dict(h=num(L, 278), vwc_of_h=bc["volumetric_water_content"] + bc["theta_r"])))
    K.append(case("head_brooks_corey_neg_lambda", "head_brooks_corey", f"{L}:282-292", dict(bc, c=num(L, 283)),
                  dict(h=bc["air_entry_pressure"], vwc_of_h=bc["theta_s"]), cmp="h_exact"))
    h3h, h3l = num(L, 296), num(L, 297)
    for i, (ln, exp) in enumerate([(300, h3l), (304, (h3h + h3l) / 2), (308, h3h)]):
        K.append(case(f"feddes_h3_{i}", "feddes_h3", f"{L}:{ln}-{ln + 1}",
                      dict(h3_high=h3h, h3_low=h3l, tpot=num(L, ln)), dict(h3=exp),
                      cmp="exact" if i == 0 else "approx"))
    fh = dict(h1=num(L, 311), h2=num(L, 312), h3=num(L, 313), h4=num(L, 314))
    rw = [(317, 320, 0.0), (317, 324, 1.4 / 1.47), (317, 328, 1.0), (317, 332, 4 / 9), (317, 336, 0.0),
          (340, 343, 0.0), (340, 347, 1.4 / 1.47), (340, 351, 1.0), (340, 355, 1.0), (340, 359, 1.0)]
    for i, (la, lh, exp) in enumerate(rw):
        K.append(case(f"rwu_feddes_{i}", "rwu_reduction_feddes", f"{L}:{lh}-{lh + 1}",
                      dict(fh, alpha_h1=num(L, la), h=num(L, lh)), dict(alpha=exp)))
    K.append(case("soil_temperature", "soil_temperature", f"{L}:363-368",
                  dict(tsoil_prev=num(L, 364), w_soil=num(L, 365), temperature=num(L, 366)),
                  dict(tsoil=num(L, 367))))
    irf = dict(soil_surface_temperature=num(L, 371), cf_soil=num(L, 372), modelsnow=1)
    K.append(case("infiltration_reduction_on", "infiltration_reduction_factor", f"{L}:375-382",
                  dict(irf, soil_infiltration_reduction=1), dict(f=num(L, 382))))
    K.append(case("infiltration_reduction_off", "infiltration_reduction_factor", f"{L}:384-391",
                  dict(irf, soil_infiltration_reduction=0), dict(f=1.0), cmp="exact"))
    eu = dict(potential_soilevaporation=num(L, 395), unsaturated_layer_depth=num(L, 396),
              unsaturated_layer_thickness=num(L, 397), water_table_depth=num(L, 398), theta_effective=num(L, 399))
    K.append(case("soilevap_unsat_0", "soil_evaporation_unsaturated_store", f"{L}:401-410",
                  dict(eu, n_unsatlayers=0), dict(e=0.0), cmp="exact"))
    K.append(case("soilevap_unsat_1", "soil_evaporation_unsaturated_store", f"{L}:412-421",
                  dict(eu, n_unsatlayers=1), dict(e=num(L, 421))))
    K.append(case("soilevap_unsat_2", "soil_evaporation_unsaturated_store", f"{L}:423-432",
                  dict(eu, n_unsatlayers=2), dict(e=num(L, 432))))
    es = dict(dt=num(L, 436), potential_soilevaporation=num(L, 438), layerthickness=num(L, 439),
              water_table_depth=num(L, 440), theta_effective=num(L, 441))
    K.append(case("soilevap_sat_0", "soil_evaporation_saturated_store", f"{L}:443-452",
                  dict(es, n_unsatlayers=0), dict(e=num(L, 452)),
                  note="the reference expects a negative value here"))
    K.append(case("soilevap_sat_2", "soil_evaporation_saturated_store", f"{L}:454-463",
                  dict(es, n_unsatlayers=2), dict(e=0.0), cmp="exact"))
    ai = dict(potential_infiltration=num(L, 467), compacted_soil_area_fraction=num(L, 469),
              infiltration_capacity_soil=num(L, 470), infiltration_capacity_compacted_soil=num(L, 471),
              f_infiltration_reduction=num(L, 472))
    K.append(case("actual_infiltration_soil_path_pos", "actual_infiltration_soil_path", f"{L}:474-486",
                  dict(ai, actual_infiltration=num(L, 475)),
                  dict(actual_infiltration_soil=num(L, 485), actual_infiltration_compacted_soil=num(L, 486))))
    K.append(case("actual_infiltration_soil_path_zero", "actual_infiltration_soil_path", f"{L}:488-500",
                  dict(ai, actual_infiltration=num(L, 489)),
                  dict(actual_infiltration_soil=0.0, actual_infiltration_compacted_soil=0.0), cmp="exact"))
    # ------------------------------------------------------------------------ soil.jl
    K.append(case("update_bc_soil_model", "update_bc_soil_model", f"{S}:1-64",
                  dict(soil=dict(soil_fraction=num(S, 8)), potential_evaporation=num(S, 10),
                       canopy_potevap=num(S, 29), interception_rate=num(S, 30), water_flux_surface=num(S, 42),
                       runoff_land=num(S, 37), runoff_river=num(S, 38)),
                  dict(potential_transpiration=num(S, 60), potential_soilevaporation=num(S, 62),
                       water_flux_surface=num(S, 63))))
    K.append(case("unsaturated_zone_flow", "unsaturated_zone_flow", f"{S}:66-106",
                  dict(dt=num(S, 68), soil=dict(
                      maximum_number_of_layers=6,
                      unsaturated_layer_thickness=nums(S, 78)[:6],
                      unsaturated_layer_depth=nums(S, 81)[:6],
                      n_unsatlayers=int(num(S, 83)), theta_s=num(S, 84), theta_r=num(S, 85),
                      kv_0=num(S, 86, 0), f=num(S, 86, 1),
                      kv_factor=nums(S, 87)[:6],
                      brooks_corey_exponent=span(S, 90, 95),
                      infiltration=num(S, 98))),
                  dict(unsaturated_layer_depth=nums(S, 104)[:6], transfer=num(S, 105))))
    K.append(case("soil_evaporation", "soil_evaporation", f"{S}:108-137",
                  dict(dt=num(S, 112), soil=dict(
                      maximum_number_of_layers=6, potential_soilevaporation=num(S, 116),
                      unsaturated_layer_thickness=nums(S, 118)[:6],
                      unsaturated_layer_depth=nums(S, 121)[:6],
                      n_unsatlayers=int(num(S, 123)), water_table_depth=num(S, 124), theta_s=num(S, 125),
                      theta_r=num(S, 126), theta_fc=num(S, 127), actual_layer_thickness=nums(S, 128)[:6],
                      drainable_water_depth=num(S, 129))),
                  dict(soil_evaporation_saturated_zone=0.0, soil_evaporation=num(S, 135),
                       drainable_water_depth=num(S, 136))))
    K.append(case("transpiration", "transpiration", f"{S}:139-190",
                  dict(dt=num(S, 141), soil=dict(
                      maximum_number_of_layers=4, h3_high=num(S, 148), h3_low=num(S, 149),
                      potential_transpiration=num(S, 150), n_unsatlayers=int(num(S, 151)),
                      water_table_depth=num(S, 152), unsaturated_layer_thickness=nums(S, 153)[:4],
                      unsaturated_layer_depth=nums(S, 155)[:4], rooting_depth=num(S, 157),
                      rootfraction=nums(S, 159)[:4], actual_layer_thickness=nums(S, 161)[:4],
                      cumulative_layer_depth=nums(S, 162)[:5], brooks_corey_exponent=span(S, 165, 168),
                      theta_s=num(S, 171), theta_r=num(S, 172), air_entry_pressure=num(S, 173), h1=num(S, 174),
                      h2=num(S, 175), h3=num(S, 176), h4=num(S, 177), alpha_h1=num(S, 178),
                      wet_root_distribution_parameter=num(S, 179), drainable_water_depth=num(S, 180))),
                  dict(actual_evaporation_unsaturated_store=num(S, 186), actual_evaporation_saturated_zone=num(S, 187),
                       drainable_water_depth=num(S, 188), transpiration=num(S, 189))))
    K.append(case("capillary_flux", "capillary_flux", f"{S}:192-228",
                  dict(dt=num(S, 196), soil=dict(
                      maximum_number_of_layers=6, rooting_depth=num(S, 200), n_unsatlayers=int(num(S, 201)),
                      kv_0=num(S, 202, 0), f=num(S, 202, 1), kv_factor=nums(S, 203)[:6],
                      water_table_depth=num(S, 204), unsaturated_layer_thickness=nums(S, 205)[:6],
                      unsaturated_layer_depth=span(S, 208, 213),
                      actual_evaporation_unsaturated_store=num(S, 216), unsaturated_store_capacity=num(S, 217),
                      drainable_water_depth=num(S, 218), cap_hmax=num(S, 219), cap_n=num(S, 220),
                      theta_s=num(S, 221), theta_r=num(S, 222))),
                  dict(actual_capillary_flux=num(S, 227))))
    K.append(case("update_soil_water_storage", "update_soil_water_storage", f"{S}:230-309",
                  dict(dt=num(S, 233), exfiltwater_average=num(S, 291), runoff_land=num(S, 280, 0),
                       actual_open_water_evaporation_land=num(S, 280, 1), soil=dict(
                      maximum_number_of_layers=4, runoff=num(S, 239), water_table_depth=num(S, 240),
                      unsaturated_layer_thickness=nums(S, 241)[:4], unsaturated_layer_depth=span(S, 244, 247),
                      n_unsatlayers=int(num(S, 250)), volumetric_water_content=span(S, 253, 256),
                      relative_volumetric_water_content=nums(S, 260)[:4], number_of_layers=int(num(S, 262)),
                      actual_layer_thickness=nums(S, 263)[:4], theta_s=num(S, 264), theta_r=num(S, 265),
                      theta_fc=num(S, 266), rooting_depth=num(S, 267), cumulative_layer_depth=nums(S, 268)[:5],
                      soil_thickness=num(S, 269), soil_water_capacity=num(S, 270),
                      unsaturated_store_capacity=num(S, 271), saturated_water_depth=num(S, 272),
                      drainable_water_depth=num(S, 273), total_soil_water_storage=num(S, 274),
                      saturation_excess_water=num(S, 275), infiltration_excess=num(S, 276))),
                  dict(runoff=num(S, 296), unsaturated_store_capacity=num(S, 297), saturated_water_depth=num(S, 298),
                       drainable_water_depth=num(S, 299), exfiltration_saturated_water=num(S, 300),
                       volumetric_water_content=nums(S, 302)[:4], relative_volumetric_water_content=nums(S, 304)[:4],
                       volumetric_water_content_root_zone=num(S, 305),
                       relative_volumetric_water_content_root_zone=num(S, 307),
                       total_soil_water_storage=num(S, 308))))
    # -------------------------------------------------------------- routing_process.jl
    kw = dict(alpha=num(R, 2), dt=num(R, 3), dx=num(R, 4))
    K.append(case("kinematic_wave", "kinematic_wave", f"{R}:1-13",
                  dict(kw, q_in=num(R, 7), q_prev=num(R, 8), q_lat=num(R, 9)),
                  dict(q=num(R, 12), crossarea=num(R, 13))))
    K.append(case("kinematic_wave_zero", "kinematic_wave", f"{R}:15-19",
                  dict(kw, q_in=num(R, 16), q_prev=num(R, 17), q_lat=num(R, 18)),
                  dict(q=0.0, crossarea=0.0), cmp="exact"))
    cel = dict(water_table_depth=num(R, 23), theta_e=num(R, 24), slope=num(R, 25), kh_0=num(R, 29, 0),
               f=num(R, 29, 1))
    K.append(case("ssf_celerity_exp", "ssf_celerity", f"{R}:28-31", dict(cel, profile=0, z_exp=0.0),
                  dict(celerity=num(R, 31))))
    K.append(case("ssf_celerity_expconst", "ssf_celerity", f"{R}:33-36", dict(cel, profile=1, z_exp=num(R, 34)),
                  dict(celerity=num(R, 36))))
    K.append(case("kw_ssf_newton_raphson", "kw_ssf_newton_raphson", f"{R}:39-48",
                  dict(q=num(R, 40), constant_term=num(R, 41), celerity=num(R, 42), dt=num(R, 43), dx=num(R, 44)),
                  dict(q=num(R, 47))))
    soil_a = dict(maximum_number_of_layers=4, number_of_layers=4, actual_layer_thickness=nums(R, 107)[:4],
                  cumulative_layer_depth=nums(R, 108)[:5], theta_s=num(R, 111), theta_r=num(R, 112),
                  theta_fc=num(R, 113), unsaturated_layer_thickness=nums(R, 133)[:4],
                  unsaturated_layer_depth=nums(R, 135)[:4], n_unsatlayers=int(num(R, 137)),
                  water_table_depth=num(R, 138))
    ssf = dict(q_in=num(R, 114), q_prev=num(R, 116), zi_prev=num(R, 117), q_net=num(R, 118), slope=num(R, 119),
               sy=num(R, 120), d=num(R, 121), dt=num(R, 122), dx=num(R, 123), dw=num(R, 124), q_max=num(R, 125),
               kh_0=num(R, 126, 0), f=num(R, 126, 1), profile=0, z_exp=0.0)
    K.append(case("kinematic_wave_ssf_its", "kinematic_wave_ssf", f"{R}:149-170", dict(ssf, soil=soil_a),
                  dict(q=num(R, 167), water_table_depth=num(R, 168), exfilt=num(R, 169), net_flux=num(R, 170))))
    K.append(case("kinematic_wave_ssf_dry", "kinematic_wave_ssf", f"{R}:172-197",
                  dict(ssf, q_prev=num(R, 173), q_net=num(R, 174), zi_prev=num(R, 175), soil=soil_a),
                  dict(q=0.0, water_table_depth=ssf["d"], exfilt=0.0, net_flux=0.0), cmp="exact"))
    soil_b = dict(soil_a, unsaturated_layer_thickness=nums(R, 203)[:4], unsaturated_layer_depth=nums(R, 205)[:4],
                  n_unsatlayers=int(num(R, 207)), water_table_depth=num(R, 208))
    K.append(case("kinematic_wave_ssf_expconst", "kinematic_wave_ssf", f"{R}:199-252",
                  dict(ssf, q_prev=num(R, 219), zi_prev=num(R, 220), q_net=num(R, 221), slope=num(R, 222),
                       sy=num(R, 223), d=num(R, 224), dt=num(R, 225), dx=num(R, 226), dw=num(R, 227),
                       q_max=num(R, 228), profile=1, z_exp=num(R, 229), soil=soil_b),
                  dict(q=num(R, 249), water_table_depth=num(R, 250), exfilt=num(R, 251), net_flux=num(R, 252))))
    riv = dict(flow_width=nums(R, 300)[:2], flow_length=nums(R, 301)[:2], alpha=nums(R, 343)[:2],
               q=nums(R, 350)[:2], p=0.05,
               reservoir=dict(external_inflow=num(R, 313), precipitation=num(R, 314), evaporation=num(R, 315),
                              inflow_overland=num(R, 316), inflow_subsurface=num(R, 317), area=num(R, 323),
                              maximum_release=num(R, 324), demand=num(R, 325),
                              target_minimum_fraction=num(R, 326), target_full_fraction=num(R, 327),
                              maximum_storage=num(R, 328), waterlevel=num(R, 331), storage=num(R, 332),
                              outflow_type=4))
    K.append(case("river_stable_timestep_and_update", "kinwave_river_update", f"{R}:290-383", riv,
                  dict(dt=num(R, 372), q=nums(R, 373)[:2], h=nums(R, 374)[:2], storage=nums(R, 375)[:2],
                       q_cumulative=nums(R, 376)[:2], reservoir_waterlevel=num(R, 379),
                       reservoir_storage=num(R, 380), reservoir_outflow=num(R, 381),
                       reservoir_actevap_cumulative=num(R, 382)),
                  note="node 1 carries a simple reservoir (outflow type 4, linear storage profile) with an "
                       "abstraction; node 2 receives its outflow (the test's upstream list also keeps node 1)"))
    # accucapacityflux on the 6-node graph of the PCRaster accucapacity example (exact)
    edges = [nums(R, ln)[-2:] for ln in range(261, 266)]
    ds = [-1] * 6
    for a, b in edges:
        ds[int(a) - 1] = int(b) - 1
    dt_acc = num(R, 269)
    K.append(case("accucapacityflux_1", "accucapacityflux", f"{R}:255-277",
                  dict(downstream=ds, order=list(range(6)), dt=dt_acc, material=[dt_acc * v for v in nums(R, 270)],
                       capacity=[nums(R, 271)[0]] * 6),
                  dict(material=[dt_acc * v for v in nums(R, 274)], flux=nums(R, 275)), cmp="exact"))
    K.append(case("accucapacityflux_2", "accucapacityflux", f"{R}:279-287",
                  dict(downstream=ds, order=list(range(6)), dt=dt_acc, material=[dt_acc * nums(R, 280)[0]] * 6,
                       capacity=nums(R, 281)),
                  dict(material=[dt_acc * v for v in nums(R, 284)], flux=nums(R, 285)), cmp="exact"))
    # local-inertial flow (surface_process.jl:88-163), both cross-sections
    K.append(case("local_inertial_flow_area", "local_inertial_flow_area", f"{R}:1320-1344",
                  dict(q0=num(R, 1322), zs0=num(R, 1323), zs1=num(R, 1324), hf=num(R, 1325), A=num(R, 1326),
                       R=num(R, 1327), length=num(R, 1328), mannings_n_sq=num(R, 1329), froude_limit=1,
                       dt=num(R, 1331)),
                  dict(q=num(R, 1344))))
    K.append(case("local_inertial_flow_rect", "local_inertial_flow_rect", f"{R}:1346-1373",
                  dict(theta=num(R, 1347), q0=num(R, 1348), qd=num(R, 1349), qu=num(R, 1350), zs0=num(R, 1351),
                       zs1=num(R, 1352), hf=num(R, 1353), width=num(R, 1354), length=num(R, 1355),
                       mannings_n_sq=num(R, 1356), froude_limit=1, dt=num(R, 1358)),
                  dict(q=num(R, 1373))))
    # 2D overland local-inertial flow at an edge, and the water depth update of land and river
    # cells (1-based index lists as in the reference's test)
    K.append(case("li_directional_flow", "li_directional_flow", f"{R}:989-1048",
                  dict(i=int(num(R, 1040)), ywidth_e=nums(R, 1002), zx_max_e=nums(R, 1004), theta=num(R, 1005),
                       h_thresh=num(R, 1006), nsq_e=span(R, 1009, 1011), z=nums(R, 1013), qx=nums(R, 1019),
                       h=nums(R, 1020), ind_x_up=nums(R, 1029), ind_x_down=nums(R, 1030), x_length=nums(R, 1034),
                       y_length=nums(R, 1035), river_location=nums(R, 1036), alpha=num(R, 995)),
                  dict(dt=num(R, 1044), qx_i=num(R, 1047))))
    K.append(case("li_water_depth", "li_water_depth", f"{R}:1050-1187",
                  dict(qx=nums(R, 1060), qy=nums(R, 1061), storage=nums(R, 1062), h=nums(R, 1063),
                       runoff=nums(R, 1067), bankfull_storage=nums(R, 1096)[0], bankfull_depth=nums(R, 1097)[0],
                       q_river=nums(R, 1106), h_river=nums(R, 1109)[0], storage_river=nums(R, 1110)[0],
                       ind_x_down=nums(R, 1121), ind_y_down=nums(R, 1122), x_length=nums(R, 1126),
                       y_length=nums(R, 1127), river_width=nums(R, 1135)[0], river_length=nums(R, 1136)[0],
                       alpha=num(R, 1085)),
                  dict(dt=num(R, 1142), storage_change=num(R, 1152), external_inflow=[0.0, 0.0],
                       depths=[num(R, 1156), num(R, 1157), num(R, 1158)], land_storage_change=num(R, 1181),
                       land_storage=num(R, 1185), land_h=num(R, 1186)),
                  note="river cell 1 sits on land cell 3 with river edge 1 in and edge 2 out"))
    # the long channel of MacDonald (1997) run to steady state with the local-inertial river
    K.append(case("local_inertial_macdonald", "local_inertial_macdonald", f"{R}:1189-1318",
                  dict(L=num(R, 1195), dx=num(R, 1196), width=nums(R, 1225)[0], mannings_n=nums(R, 1226)[0],
                       h_thresh=num(R, 1265), alpha=num(R, 1270), epsilon=num(R, 1303), inflow=num(R, 1306)),
                  dict(mean_abs_error=num(R, 1317)),
                  note="bed levels integrate the analytical slope (the test's quadgk, rtol 1e-12); "
                       "the analytical depth profile is MacDonald's (1997), restated from lines 1199-1211"))
    # -------------------------------------------------------------------- reservoir.jl
    # update_reservoir_model!(res, i, inflow, dt) of one reservoir after set_reservoir_vars!
    # (reservoir.jl:583-628), and the river-side wrapper that limits the abstraction and hands
    # the outflow to the downstream cell (surface_kinwave.jl:441-489). The linked-reservoir and
    # rating-curve tests read CSV tables that the checkout does not hold.
    V = "reservoir.jl"
    simple = dict(outflow_type=4, precipitation=num(V, 9), evaporation=num(V, 10), demand=num(V, 14),
                  maximum_release=num(V, 15), maximum_storage=num(V, 16), area=num(V, 17),
                  target_full_fraction=num(V, 18), target_minimum_fraction=num(V, 19), storage=num(V, 25),
                  waterlevel=num(V, 26))
    K.append(case("reservoir_simple", "update_reservoir_model", f"{V}:1-44",
                  dict(reservoir=simple, inflow=num(V, 36), dt=num(V, 4)),
                  dict(outflow=num(V, 38), storage=num(V, 40), actevap_cumulative=num(V, 43))))
    K.append(case("reservoir_simple_observed_outflow", "update_reservoir_model", f"{V}:46-57",
                  dict(reservoir=dict(simple, outflow_obs=num(V, 47), storage=num(V, 48), waterlevel=num(V, 49)),
                       inflow=num(V, 52), dt=num(V, 4)),
                  dict(outflow=num(V, 54), storage=num(V, 56))))
    K.append(case("reservoir_modified_puls", "update_reservoir_model", f"{V}:60-115",
                  dict(reservoir=dict(outflow_type=3, precipitation=num(V, 68), evaporation=num(V, 69),
                                      area=num(V, 73), threshold=num(V, 74), rating_curve_coefficient=num(V, 77),
                                      rating_curve_exponent=num(V, 78), waterlevel=num(V, 80),
                                      storage=num(V, 73) * num(V, 80)),
                       inflow=num(V, 100), dt=num(V, 65)),
                  dict(waterlevel=num(V, 107), outflow=num(V, 108), storage=num(V, 110),
                       actevap_cumulative=num(V, 114)),
                  note="initialize_storage of the linear profile: storage = area * waterlevel"))
    K.append(case("reservoir_observed_outflow_at_node", "update_reservoir_at_node", f"{V}:117-167",
                  dict(reservoir=dict(outflow_type=4, external_inflow=num(V, 127), inflow_overland=num(V, 128),
                                      inflow_subsurface=num(V, 129), precipitation=num(V, 130),
                                      evaporation=num(V, 131), area=num(V, 137), threshold=num(V, 138),
                                      rating_curve_coefficient=num(V, 139), rating_curve_exponent=num(V, 140),
                                      waterlevel=num(V, 143), storage=num(V, 144), outflow_obs=num(V, 147)),
                       q=nums(V, 152)[-2], dt=num(V, 159)),
                  dict(qin_downstream=num(V, 162), abstraction_cumulative=num(V, 163), storage=num(V, 164),
                       waterlevel=num(V, 165), outflow=num(V, 166))))
    K.append(case("reservoir_simple_at_node", "update_reservoir_at_node", f"{V}:169-221",
                  dict(reservoir=dict(outflow_type=4, external_inflow=num(V, 178), inflow_overland=num(V, 179),
                                      inflow_subsurface=num(V, 180), precipitation=num(V, 181),
                                      evaporation=num(V, 182), area=num(V, 188), maximum_release=num(V, 189),
                                      demand=num(V, 190), target_minimum_fraction=num(V, 191),
                                      target_full_fraction=num(V, 192), maximum_storage=num(V, 193),
                                      waterlevel=num(V, 196), storage=num(V, 197)),
                       q=nums(V, 204)[0], dt=num(V, 212)),
                  dict(qin_downstream=num(V, 215), abstraction_cumulative=num(V, 217), storage=num(V, 218),
                       waterlevel=num(V, 219), outflow=num(V, 220))))
    # ------------------------------------------------------------------------ utils.jl
    # units (the file helpers' conversions) and the affine transform of [input] entries
    K.append(case("units_absolute_degrees", "to_si", f"{U}:40-45", dict(value=0.0, unit="degC"),
                  dict(si=num(U, 44)), cmp="exact"))
    K.append(case("units_per_step", "to_si_factor_per_step", f"{U}:51-54", dict(dt=num(U, 51)),
                  dict(factor=1.0 / num(U, 51)), cmp="exact",
                  note="to_SI_factor(Unit(m = 1, dt = -1); dt_val = dt) == inv(dt)"))
    v = nums(U, 294)
    K.append(case("affine_scale", "affine", f"{U}:291-296", dict(v=v, scale=nums(U, 296)[:1]),
                  dict(out=[nums(U, 296)[0] * x for x in v]), cmp="exact"))
    K.append(case("affine_scale_offset", "affine", f"{U}:291-305", dict(v=v, scale=[6.0], offset=[7.0] * 3),
                  dict(out=[6.0 * x + 7.0 for x in v]), cmp="exact",
                  note="scale = [6.0], offset = fill(7.0, 3) (utils.jl:301-304)"))
    # julian_day (leap days not counted): the standard-calendar cases
    for ln in range(19, 28):
        y, mo, d, day = nums(U, ln)[:4]
        K.append(case(f"julian_day_{int(y)}_{int(mo):02d}_{int(d):02d}", "julian_day", f"{U}:{ln}",
                      dict(year=int(y), month=int(mo), day=int(d)), dict(julian_day=int(day)), cmp="exact"))
    K.append(case("scurve", "scurve", f"{U}:66-77",
                  dict(x=num(U, 71), a=num(U, 67), b=num(U, 68), c=num(U, 69)), dict(s=num(U, 73))))
    K.append(case("mass_balance_zero", "compute_mass_balance_error", f"{U}:105-112",
                  dict(total_in=num(U, 106), total_out=num(U, 107), storage_rate=num(U, 108)),
                  dict(error=0.0, relative_error=0.0), cmp="exact"))
    K.append(case("mass_balance_nonzero", "compute_mass_balance_error", f"{U}:114-118",
                  dict(total_in=num(U, 106), total_out=num(U, 114), storage_rate=num(U, 108)),
                  dict(error=-1.0, relative_error=-2 / 11), cmp="error_exact"))
    wt_soil = dict(maximum_number_of_layers=5, unsaturated_layer_depth=nums(U, 255)[:5],
                   unsaturated_layer_thickness=nums(U, 257)[:5], theta_s=num(U, 260), theta_r=num(U, 261),
                   n_unsatlayers=int(num(U, 262)))
    K.append(case("water_table_change_falling", "water_table_change", f"{U}:265-269",
                  dict(dt=num(U, 246), specific_yield=num(U, 249), net_flux=num(U, 266), soil=wt_soil),
                  dict(dh=num(U, 268), exfilt=0.0)))
    K.append(case("water_table_change_rising", "water_table_change", f"{U}:271-276",
                  dict(dt=num(U, 246), specific_yield=num(U, 249), net_flux=num(U, 273), soil=wt_soil),
                  dict(dh=num(U, 275), exfilt=0.0)))
    return K


if __name__ == "__main__":
    kats = build()
    OUT.write_text(json.dumps({"source": "Wflow.jl 1.1.0-dev unit tests (Wflow/test)",
                               "rtol_approx": 1.4901161193847656e-08, "cases": kats}, indent=1) + "\n")
    print(f"wrote {len(kats)} cases to {OUT}")
