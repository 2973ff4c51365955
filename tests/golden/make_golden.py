"""Extract the golden fixtures of the WCSPH path from the reference tree.

Run in a container where the reference is present:
    python tests/golden/make_golden.py /path/to/TrixiParticles.jl
Writes
* tests/golden/validation_wcsph_40.json: the series of the reference's own 2D dam-break
  validation run (validation/dam_break_2d/validation_reference_wcsph_40.json, produced by the
  reference with SerialUpdate on an x86 CPU) together with the run parameters from its `meta`
  block and from validation/dam_break_2d/setup_marrone_2011.jl + examples/fluid/dam_break_2d.jl;
* tests/golden/rectangular_tank_faces.json: the expected wall coordinates of the reference's
  "Boundary Faces" test (test/setups/rectangular_tank.jl:185-270), one and three layers for
  every face selection, read from the Julia matrix literals of that file;
* tests/golden/rectangular_tank_coordinates.json: the expected fluid and wall coordinates of its
  "Coordinates" tests in 2D and 3D (one layer for two spacings, two spacing ratios and two
  corners; three layers), test/setups/rectangular_tank.jl:1-58, 125-141, 274-340, 373-387;
* tests/golden/rectangular_shape_coordinates.json: the expected coordinates of the "Positions"
  and "Loop Orders" tests of test/setups/rectangular_shape.jl (2D: 1-52, 3D: 193-240).
"""
import json
import re
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
    tank_faces(ref_root)
    tank_coordinates(ref_root)
    shape_coordinates(ref_root)


def shape_coordinates(ref_root: str) -> None:
    src = (Path(ref_root) / "test" / "setups" / "rectangular_shape.jl").read_text()
    cases = []
    for nd, text in ((2, src[src.index('"Rectangular Shape 2D"'):
                             src.index('"Rectangular Shape 3D"')]),
                     (3, src[src.index('"Rectangular Shape 3D"'):])):
        pos = text[text.index('"Positions"'):text.index('"Loop Orders"')]
        corners = [[float(x) for x in t.split(",")] for t in
                   re.findall(r"\(([-0-9., ]+)\)", pos[pos.index("positions = ["):
                                                   pos.index("expected_coords")])]
        spacing = float(re.search(r"particle_spacing = ([0-9.]+)", pos).group(1))
        n = [int(x) for x in re.search(r"n_particles_per_dimension = \(([0-9, ]+)\)",
                                        pos).group(1).split(",")]
        exp = _julia_array(pos[pos.index("expected_coords = ["):])
        assert len(corners) == len(exp)
        for corner, coords in zip(corners, exp):
            cases.append({"ndims": nd, "particle_spacing": spacing, "n": n,
                          "min_coordinates": corner, "loop_order": "x_first",
                          "place_on_shell": False, "coordinates": coords})
        lo = text[text.index('"Loop Orders"'):text.index('"Incompressible Hydrostatic Pressure"')]
        orders = re.findall(r":(\w+_first)", lo[lo.index("loop_orders = ["):
                                                lo.index("expected_coords")])
        exp = _julia_array(lo[lo.index("expected_coords = ["):])
        assert len(orders) == len(exp)
        for order, coords in zip(orders, exp):
            cases.append({"ndims": nd, "particle_spacing": 1.0, "n": [2] * nd,
                          "min_coordinates": [0.0] * nd, "loop_order": order,
                          "place_on_shell": True, "coordinates": coords})
    out = {"source": "test/setups/rectangular_shape.jl (Positions, Loop Orders)",
           "cases": cases}
    (HERE / "rectangular_shape_coordinates.json").write_text(json.dumps(out))


def _julia_array(text: str):
    """A Julia array literal at the start of `text` (after its opening bracket is found) as nested
    lists: `[a b; c d]` (rows split at `;` or a line break) -> list of rows, `[[..], [..]]` -> list
    of the inner literals.  Comments are dropped."""
    text = re.sub(r"#[^\n]*", "", text)
    pos = text.index("[")

    def parse(i):
        j = i + 1
        while text[j] in " \t\n":
            j += 1
        if text[j] == "[":  # a vector of arrays
            items = []
            while True:
                while text[j] in " \t\n,":
                    j += 1
                if text[j] == "]":
                    return items, j + 1
                item, j = parse(j)
                items.append(item)
        k = text.index("]", j)
        rows = [r.split() for r in re.split(r"[;\n]", text[j:k])]
        return [[float(x) for x in r] for r in rows if r], k + 1

    return parse(pos)[0]


def tank_coordinates(ref_root: str) -> None:
    src = (Path(ref_root) / "test" / "setups" / "rectangular_tank.jl").read_text()
    cases = []

    def section(start, end):
        a = src.index(start)
        return src[a:src.index(end, a)]

    def one_layer(text, nd, fluid, tank, corners):
        fl = _julia_array(text[text.index("expected_fluid_coords = ["):])
        bd = _julia_array(text[text.index("expected_bound_coords = ["):])
        for corner in corners:
            for j, dx in enumerate((0.1, 0.2)):
                for k, ratio in enumerate((1, 3)):
                    cases.append({"ndims": nd, "particle_spacing": dx, "fluid_size": fluid,
                                  "tank_size": tank, "fluid_density": 1000.0, "n_layers": 1,
                                  "spacing_ratio": ratio, "min_coordinates": corner,
                                  "fluid_coordinates": fl[j],
                                  "boundary_coordinates": bd[j][k]})

    def three_layers(text, nd):
        bd = _julia_array(text[text.index("expected_bound_coords = ["):])
        cases.append({"ndims": nd, "particle_spacing": 0.5, "fluid_size": [0.5] * nd,
                      "tank_size": [1.0] * nd, "fluid_density": 500.0, "n_layers": 3,
                      "spacing_ratio": 1, "min_coordinates": [0.0] * nd,
                      "fluid_coordinates": None, "boundary_coordinates": bd})

    d2 = section('"Rectangular Tank 2D"', '"Rectangular Tank 3D"')
    d3 = src[src.index('"Rectangular Tank 3D"'):]
    one_layer(section('"Rectangular Tank 2D"', '"Velocities"'), 2, [0.5, 0.4],
              [0.5, 0.5], ([0.0, 0.0], [-0.3, 2.0]))
    three_layers(d2[d2.index('"Multiple Boundary Layers"'):], 2)
    one_layer(d3[:d3.index('"Reset Wall"')], 3, [0.4, 0.4, 0.4], [0.4, 0.4, 0.4],
              ([0.0, 0.0, 0.0], [-0.3, 2.0, -0.5]))
    three_layers(d3[d3.index('"Multiple Boundary Layers"'):], 3)
    out = {"source": "test/setups/rectangular_tank.jl (Coordinates testsets)",
           "note": "coordinates before the shift to min_coordinates, as in the reference test",
           "cases": cases}
    (HERE / "rectangular_tank_coordinates.json").write_text(json.dumps(out))


def _julia_matrices(text: str) -> list:
    """The 2-row matrices `[a b ...; c d ...]` of a Julia vector literal `[ [..], [..] ]`, as
    lists of rows."""
    body = text[text.index("[") + 1:]
    out, depth, cur = [], 0, ""
    for ch in body:
        if ch == "[":
            depth += 1
            cur = "" if depth == 1 else cur
            continue
        if ch == "]":
            if depth == 0:
                break
            depth -= 1
            if depth == 0:
                out.append([[float(x) for x in row.split()]
                            for row in cur.replace("\n", " ").split(";")])
            continue
        if depth >= 1:
            cur += ch
    return out


def tank_faces(ref_root: str) -> None:
    src = (Path(ref_root) / "test" / "setups" / "rectangular_tank.jl").read_text()
    block = src[src.index('@testset verbose=true "Boundary Faces"'):
                src.index("expected_bound_coords = (expected_bound_coords1")]
    faces_txt = block[block.index("faces = ["):block.index("# One boundary layer")]
    faces = [[x == "true" for x in re.findall(r"true|false", f)]
             for f in re.findall(r"\(([^)]*)\)", faces_txt)]
    one = _julia_matrices(block[block.index("expected_bound_coords1 = ["):])
    three = _julia_matrices(block[block.index("expected_bound_coords2 = ["):])
    assert len(faces) == len(one) == len(three) == 14
    out = {
        "source": "test/setups/rectangular_tank.jl:185-270",
        "tank": {"particle_spacing": 0.2, "fluid_size": [0.6, 0.6], "tank_size": [0.8, 0.8],
                 "fluid_density": 750.5},
        "cases": [{"n_layers": n, "faces": f, "boundary_coordinates": m}
                  for n, mats in ((1, one), (3, three)) for f, m in zip(faces, mats)],
    }
    (HERE / "rectangular_tank_faces.json").write_text(json.dumps(out))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the TrixiParticles.jl source tree>")
    main(sys.argv[1])
