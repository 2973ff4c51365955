"""Extract the golden fixtures of the WCSPH path from the reference tree.

Run in a container where the reference is present:
    python tests/golden/make_golden.py /path/to/TrixiParticles.jl
Writes tests/golden/validation_wcsph_40.json: the series of the reference's own 2D dam-break
validation run (validation/dam_break_2d/validation_reference_wcsph_40.json, produced by the
reference with SerialUpdate on an x86 CPU) together with the run parameters from its `meta`
block and from validation/dam_break_2d/setup_marrone_2011.jl + examples/fluid/dam_break_2d.jl.
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(ref_root: str) -> None:
    src = Path(ref_root) / "validation" / "dam_break_2d" / "validation_reference_wcsph_40.json"
    d = json.loads(src.read_text())
    meta = d["meta"]
    ti = meta["simulation_info"]["time_integrator"]
    fl = meta["system_data"]["fluid_1"]
    bd = meta["system_data"]["boundary_1"]
    out = {
        "source": "validation/dam_break_2d/validation_reference_wcsph_40.json",
        "solver_version": meta["simulation_info"]["solver_version"],
        "params": {
            "H": 0.6,
            "W": 1.2,
            "particle_spacing": fl["particle_spacing"],
            "tank_size_formula": "floor(5.366*H/dx)*dx x 4.0",
            "n_layers": 4,
            "smoothing_length": fl["smoothing_length"],
            "sound_speed": fl["sound_speed"],
            "exponent": fl["state_equation"]["exponent"],
            "reference_density": fl["state_equation"]["reference_density"],
            "alpha": fl["viscosity_model"]["alpha"],
            "beta": fl["viscosity_model"]["beta"],
            "epsilon": fl["viscosity_model"]["epsilon"],
            "delta": fl["density_diffusion"]["delta"],
            "acceleration": fl["acceleration"],
            "wall_smoothing_length": bd["boundary_model"]["smoothing_length"],
            "wall_clip_negative_pressure": True,
            "dt_max": ti["dt_max"],
            "final_time": ti["final_time"],
            "save_interval": "0.01 / sqrt(9.81 / H)",
        },
        "series": {k: {"time": v["time"], "values": v["values"]}
                   for k, v in d.items() if k != "meta"},
    }
    (HERE / "validation_wcsph_40.json").write_text(json.dumps(out))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
