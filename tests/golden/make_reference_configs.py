"""Copy the SBM test configurations of Wflow.jl's test suite into reference_configs.json.

The TOML files are the reference's own test inputs (Wflow/test/*.toml); the configuration tests
parse them with wflow_gb300.config without needing the reference checkout at run time.

Usage: python tests/golden/make_reference_configs.py <path-to-Wflow.jl-checkout>
(or with the checkout path in the environment variable WFLOW_JL_CHECKOUT).
"""

import json
import os
import sys
from pathlib import Path

NAMES = ["sbm_config.toml", "sbm_simple.toml"]


def main():
    p = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WFLOW_JL_CHECKOUT")
    if not p:
        sys.exit("usage: make_reference_configs.py <path-to-Wflow.jl-checkout> (or set WFLOW_JL_CHECKOUT)")
    test_dir = Path(p) / "Wflow" / "test"
    out = {name: {"source": f"Wflow/test/{name}", "text": (test_dir / name).read_text()} for name in NAMES}
    dst = Path(__file__).with_name("reference_configs.json")
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(out)} configurations to {dst}")


if __name__ == "__main__":
    main()
