"""The reference's example input files (Examples/input_*.toml) as data
(tests/golden/example_configs.json, made by tests/golden/make_example_configs.py)
and a writer that turns one back into a TOML file."""
import json
import os

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "example_configs.json")
SIZES = ("Nx", "Ny", "Nz", "Nn", "Nm", "Np", "Ns", "timesteps", "dt")


def configs():
    with open(_PATH) as fh:
        return json.load(fh)


def _value(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, str):
        return '"%s"' % v
    if isinstance(v, list):
        return "[" + ", ".join(_value(x) for x in v) + "]"
    return repr(v)


def write_toml(cfg, path):
    with open(path, "w") as fh:
        for sec in ("input_parameters", "solver_parameters"):
            fh.write(f"[{sec}]\n")
            for k, v in cfg[sec].items():
                fh.write(f"{k} = {_value(v)}\n")
