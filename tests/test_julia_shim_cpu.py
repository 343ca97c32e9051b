"""The Julia binding (wflow.jl_gb300/julia/WflowGB300.jl) against the library it binds (CPU).

Julia is not installed here, so the shim cannot run; what can be checked without it is that every
symbol it calls through `ccall((:name, LIB), ...)` is exported by the built library, and that the
struct layouts it mirrors have the field counts of the C headers.
"""

import re
from pathlib import Path

from wflow_gb300 import abi, build

SHIM = Path(__file__).resolve().parents[1] / "wflow.jl_gb300" / "julia" / "WflowGB300.jl"


def test_every_ccall_symbol_is_exported():
    build.build_all()
    lib = abi.load_library(required=True)
    names = sorted(set(re.findall(r"ccall\(\(:(\w+),\s*LIB\)", SHIM.read_text())))
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_field_counts_match_the_headers():
    text = SHIM.read_text()
    for jl_name in ("WfLiLandGrid", "WfLiRiverNetwork"):
        m = re.search(r"struct %s\n(.*?)\nend" % jl_name, text, re.S)
        assert m, jl_name
        fields = [ln for ln in m.group(1).splitlines() if "::" in ln]
        from wflow_gb300 import li_river
        assert len(fields) == len(getattr(li_river, jl_name)._fields_), jl_name
    for jl_name in ("WfReservoirs", "WfReservoirTables"):
        m = re.search(r"struct %s\n(.*?)\nend" % jl_name, text, re.S)
        assert m, jl_name
        fields = [ln.split("::")[0].strip() for ln in m.group(1).splitlines() if "::" in ln]
        assert fields == [f for f, _ in getattr(abi, jl_name)._fields_], jl_name
