"""The reference's example input files through load_parameters and the
parameter set-up (spectrax/_initialization.py:14-190), on the CPU."""
import numpy as np
import pytest

from example_configs import SIZES, configs, write_toml

NAMES = sorted(configs())


@pytest.mark.parametrize("name", NAMES)
def test_example_toml_round_trip_and_setup(name, tmp_path):
    from spectrax_gb300.params import Dopri8, initialize_simulation_parameters, load_parameters
    cfg = configs()[name]
    path = tmp_path / name
    write_toml(cfg, path)
    inp, sol = load_parameters(str(path))
    for k, v in cfg["input_parameters"].items():
        assert np.allclose(inp[k], v), k
    assert isinstance(sol["solver"], Dopri8) and sol["adaptive_time_step"] is True
    p = initialize_simulation_parameters(inp, *[sol[k] for k in SIZES])
    assert p["t_max"] == cfg["input_parameters"]["t_max"]
    assert p["nabla"].shape == (3, sol["Ny"], sol["Nx"], sol["Nz"])
