"""Writes example_configs.json: the parameter sets of the reference's example
input files (Examples/input_*.toml), read as data, so that the tests can
rebuild a TOML file and run it through ``load_parameters`` without the
reference tree.  Run where the SPECTRAX source tree is available (the test
machines do not need it):

    python tests/golden/make_example_configs.py <path to the SPECTRAX source tree>
"""
import glob
import json
import os
import sys
import tomllib

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "example_configs.json")


def main(ref_root: str) -> None:
    configs = {}
    for path in sorted(glob.glob(os.path.join(ref_root, "Examples", "input_*.toml"))):
        with open(path, "rb") as fh:
            configs[os.path.basename(path)] = tomllib.load(fh)
    if not configs:
        raise SystemExit(f"no Examples/input_*.toml under {ref_root}")
    with open(OUT, "w") as fh:
        json.dump(configs, fh, indent=1, sort_keys=True)
    print(f"{len(configs)} configs -> {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_example_configs.py <path to the SPECTRAX source tree>")
    main(sys.argv[1])
