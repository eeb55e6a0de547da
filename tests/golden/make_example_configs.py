"""Writes example_configs.json: the parameter sets of the reference's example
input files (Examples/input_*.toml), read as data, so that the tests can
rebuild a TOML file and run it through ``load_parameters`` without the
reference tree.  Run here (the reference is not on the GPU machines):

    python tests/golden/make_example_configs.py
"""
import glob
import json
import os
import tomllib

REF = "/root/reference/Examples"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "example_configs.json")

configs = {}
for path in sorted(glob.glob(os.path.join(REF, "input_*.toml"))):
    with open(path, "rb") as fh:
        configs[os.path.basename(path)] = tomllib.load(fh)
with open(OUT, "w") as fh:
    json.dump(configs, fh, indent=1, sort_keys=True)
print(f"{len(configs)} configs -> {OUT}")
