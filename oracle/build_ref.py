"""Build the reference-side checkers and regenerate the golden vectors.

1. Compiles oracle/ref_kat.cpp against the reference's own vendored headers
   (external/pcg-cpp-0.98/include, external/eigen) into oracle/_ref/ref_kat
   and writes its output to tests/golden/ref_kat.json: the RNG leaves.
2. Copies the reference functions listed in SNIPPETS, each by its cited
   line range (the end found by brace matching, the first line checked
   against an anchor so that a moved line fails loudly), into
   oracle/_ref/snip/, compiles oracle/ref_pins.cpp against them into
   oracle/_ref/ref_pins, runs it on a seeded synthetic mode table and
   writes tests/golden/ref_pins.json: the flight-path functions; and on
   two smaller tables, tests/golden/ref_pins_dmm.json: the diffuse
   mismatch model between materials, with calculate_gradientT on two
   seeded geometries.

Only this script reads the reference tree, and only where it exists (the
build container); oracle/_ref/ is not committed, the fixtures it writes are,
so that tests elsewhere need no reference.

The reference tree is taken from --reference, else from the environment
variable BTE_REFERENCE_TREE, else from the build container's mount point.

Usage: python oracle/build_ref.py [--reference DIR] [--no-write]
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


_MOUNT = "/root/reference"  # where the build container mounts the reference

# (snippet, reference file, first line, anchor of the first line, line of the
# last definition whose brace-matched end closes the snippet)
SNIPPETS = [
    ("utilities_almost_equal.inc", "include/utilities.hpp", 214, "inline bool almost_equal(", 214),
    ("utilities_my_jobs.inc", "include/utilities.hpp", 343, "inline std::array<std::size_t, 2> my_jobs(", 343),
    ("utilities_bose_einstein.inc", "include/utilities.hpp", 385, "inline double bose_einstein(", 385),
    ("utilities_bose_einstein_kernel.inc", "include/utilities.hpp", 401,
     "inline double bose_einstein_kernel(", 401),
    ("particle_sign.inc", "include/deviational_particle.hpp", 27, "enum class particle_sign", 33),
    ("calc_percentiles_log.inc", "src/isotopic_scattering.cpp", 31,
     "std::array<double, 2> calc_percentiles_log(", 31),
    ("qpoint_grid_base_sigma.inc", "include/qpoint_grid.hpp", 179, "double base_sigma(", 179),
    ("sampling_hpp.inc", "include/sampling.hpp", 40, "inline double random_dt(", 303),
    ("sampling_cpp.inc", "src/sampling.cpp", 26, "void Grid_distribution::fill_cumulative(", 333),
    ("collision_error_bound.inc", "include/collision_operator.hpp", 216, "inline long double error_bound(", 216),
    ("collision_propagator_H_class.inc", "include/collision_operator.hpp", 241, "class propagator_H {", 241),
    ("collision_arnoldi.inc", "src/collision_operator.cpp", 815, "void Arnoldi_algorithm(", 815),
    ("collision_propagator_H_methods.inc", "src/collision_operator.cpp", 854, "propagator_H::propagator_H() {", 918),
    ("collision_save_load_build_P.inc", "src/collision_operator.cpp", 931, "void save_P(std::string fname,", 1015),
    ("rta_gamma_pdf.inc", "src/RTA_MC2D.cpp", 61, "double gamma_pdf(", 61),
    ("rta_get_bin_index.inc", "src/RTA_MC2D.cpp", 140, "inline Eigen::Index get_bin_index(", 140),
    ("rta_spectral_decomposition.inc", "src/RTA_MC2D.cpp", 150, "struct spectral_decomposition {", 150),
    ("rta_diffusive_bouncing.inc", "src/RTA_MC2D.cpp", 547, "class diffusive_bouncing {", 547),
    ("rta_process_segment_transient.inc", "src/RTA_MC2D.cpp", 699, "void process_segment(std::size_t ibox,", 699),
    ("rta_process_segment_periodic.inc", "src/RTA_MC2D.cpp", 784, "void process_segment(std::size_t ibox,", 784),
    ("rta_get_v.inc", "src/RTA_MC2D.cpp", 843, "inline Eigen::Vector2d get_v(", 843),
    ("dos_gaussian.inc", "include/dos.hpp", 28, "class Gaussian_for_DOS {", 28),
    ("sampling_hpp_dmm.inc", "include/sampling.hpp", 324, "class layer_coupling {", 402),
    ("sampling_cpp_dmm.inc", "src/sampling.cpp", 366, "double layer_coupling::get_injection_rate(", 831),
    ("geometry_calculate_gradientT.inc", "src/geometry_2d.cpp", 524,
     "Eigen::MatrixXd calculate_gradientT(std::vector<alma::geometry_2d>& sys) {", 524),
]


def _block_end(lines, start):
    """Index of the line that closes the first brace block opened at or
    after lines[start] (comments, strings and characters skipped)."""
    depth, opened, in_block = 0, False, False
    for i in range(start, len(lines)):
        s = lines[i]
        j, in_str, in_chr = 0, False, False
        while j < len(s):
            c = s[j]
            if in_block:
                if s.startswith("*/", j):
                    in_block = False
                    j += 1
            elif in_str:
                if c == "\\":
                    j += 1
                elif c == '"':
                    in_str = False
            elif in_chr:
                if c == "\\":
                    j += 1
                elif c == "'":
                    in_chr = False
            elif s.startswith("//", j):
                break
            elif s.startswith("/*", j):
                in_block = True
                j += 1
            elif c == '"':
                in_str = True
            elif c == "'":
                in_chr = True
            elif c == "{":
                depth += 1
                opened = True
            elif c == "}":
                depth -= 1
                if opened and depth == 0:
                    return i
            j += 1
    raise RuntimeError("unbalanced braces from line %d" % (start + 1))


def extract_snippets(reference: str, out_dir: str) -> None:
    os.makedirs(out_dir, exist_ok=True)
    for name, rel, first, anchor, last_def in SNIPPETS:
        with open(os.path.join(reference, rel)) as f:
            lines = f.read().split("\n")
        if not lines[first - 1].strip().startswith(anchor):
            raise RuntimeError(f"{rel}:{first} no longer starts with {anchor!r}; update SNIPPETS")
        end = _block_end(lines, last_def - 1)
        body = "\n".join(lines[first - 1:end + 1])
        with open(os.path.join(out_dir, name), "w") as f:
            f.write(f'#line {first} "{rel}"\n{body}\n')


def _write_table(path: str, n: int = 6, config: int = 100) -> None:
    """The seeded synthetic mode table of the pins: n x n q points x 6 branches."""
    sys.path.insert(0, os.path.join(REPO, "bte-barna_gb300"))
    import synth
    m = synth.mode_table(n, 3, 3, 300.0, config=config)
    n = int(m["nq"]) * int(m["nb"])
    with open(path, "w") as f:
        f.write(f"{m['nq']} {m['nb']}\n")
        for k in range(n):
            f.write(" ".join(repr(float(x)) for x in (m["omega"][k], m["vg"][3 * k], m["vg"][3 * k + 1],
                                                      m["vg"][3 * k + 2], m["w"][k])) + "\n")
        f.write(" ".join(repr(float(x)) for x in m["dq"]) + "\n")
        f.write(f"{float(m['V'])!r} {float(m['c_lat'])!r}\n")


def build_pins(reference: str) -> str:
    out_dir = os.path.join(HERE, "_ref")
    snip = os.path.join(out_dir, "snip")
    extract_snippets(reference, snip)
    exe = os.path.join(out_dir, "ref_pins")
    cmd = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w",
        "-I", snip,
        "-I", os.path.join(reference, "include"),
        "-I", os.path.join(reference, "external", "pcg-cpp-0.98", "include"),
        "-I", os.path.join(reference, "external", "eigen"),
        os.path.join(HERE, "ref_pins.cpp"), "-o", exe,
    ]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("ref_pins build failed:\n" + r.stdout + r.stderr)
    return exe


def gradient_geometries():
    """The boxes of the calculate_gradientT pins: a 20 x 10 grid with a
    staircase pore and seeded random Teq (4 to 8 neighbours per cell, corner
    contacts included), and a ribbon of 6 cells with reservoirs (collinear
    neighbours).  Returns [(geometry dict, [(centre, contacts)] per box)]."""
    sys.path.insert(0, os.path.join(REPO, "bte-barna_gb300"))
    import numpy as np
    import synth
    out = []
    g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0)
    g["Teq"] = 300.0 + np.random.default_rng(20261204).normal(0.0, 0.5, g["nboxes"])
    out.append(g)
    r = synth.ribbon_geometry(240.0, 50.0, 6)
    r["Teq"][:6] = [299.6, 299.8, 300.1, 300.2, 300.6, 300.7]
    out.append(r)
    res = []
    for g in out:
        v = np.asarray(g["vertices"], float).reshape(-1, 4, 2)
        lo, hi = v.min(axis=1), v.max(axis=1)
        c = 0.5 * (lo + hi)
        n = len(v)
        boxes = []
        for a in range(n):
            nb = [b for b in range(n) if b != a
                  and lo[b, 0] <= hi[a, 0] + 1e-9 and lo[a, 0] <= hi[b, 0] + 1e-9
                  and lo[b, 1] <= hi[a, 1] + 1e-9 and lo[a, 1] <= hi[b, 1] + 1e-9]
            boxes.append((c[a], nb))
        res.append((g, boxes))
    return res


def _write_gradient_file(path: str, g: dict, boxes) -> None:
    with open(path, "w") as f:
        f.write(f"{len(boxes)}\n")
        for i, (c, nb) in enumerate(boxes):
            f.write(f"{i} {int(g['reservoir'][i])} 0 {float(g['Teq'][i])!r} {float(c[0])!r} {float(c[1])!r} "
                    f"{len(nb)} " + " ".join(str(b) for b in nb) + "\n")


def run_pins(exe: str):
    """The pins' JSON, the diffuse mismatch pins' JSON (two 4x4 x 6 tables of
    different seeds) and the calculate_gradientT pins' JSON."""
    out_dir = os.path.dirname(exe)
    table = os.path.join(out_dir, "pins_table.txt")
    _write_table(table)
    ta, tb = os.path.join(out_dir, "pins_dmm_a.txt"), os.path.join(out_dir, "pins_dmm_b.txt")
    _write_table(ta, 4, 100)
    _write_table(tb, 4, 101)
    grads = []
    for k, (g, boxes) in enumerate(gradient_geometries()):
        gf = os.path.join(out_dir, f"pins_grad_{k}.txt")
        _write_gradient_file(gf, g, boxes)
        subprocess.run([exe, table, out_dir, ta, tb, gf], check=True, capture_output=True, text=True)
        with open(os.path.join(out_dir, "ref_pins_grad.json")) as f:
            grads.append({"Teq": [float(x) for x in g["Teq"]], **json.load(f)})
    with open(os.path.join(out_dir, "ref_pins.json")) as f:
        pins = json.load(f)
    with open(os.path.join(out_dir, "ref_pins_dmm.json")) as f:
        dmm = json.load(f)
    dmm["gradientT"] = grads
    return pins, dmm


def reference_tree():
    """The reference tree to build from, or None where it does not exist."""
    path = os.environ.get("BTE_REFERENCE_TREE", _MOUNT)
    return path if os.path.isdir(path) else None


def build(reference: str) -> str:
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "ref_kat")
    cmd = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off",
        "-I", os.path.join(reference, "external", "pcg-cpp-0.98", "include"),
        "-I", os.path.join(reference, "external", "eigen"),
        os.path.join(HERE, "ref_kat.cpp"), "-o", exe,
    ]
    subprocess.run(cmd, check=True)
    return exe


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--no-write", action="store_true")
    args = ap.parse_args()
    if args.reference is None:
        args.reference = reference_tree()
    if not args.reference or not os.path.isdir(args.reference):
        print(f"reference tree {args.reference} absent; nothing to build")
        return 0
    exe = build(args.reference)
    text = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    data = json.loads(text)
    pins, dmm = run_pins(build_pins(args.reference))
    if not args.no_write:
        for name, d in (("ref_kat.json", data), ("ref_pins.json", pins), ("ref_pins_dmm.json", dmm)):
            path = os.path.join(REPO, "tests", "golden", name)
            with open(path, "w") as f:
                json.dump(d, f, indent=1 if name == "ref_kat.json" else None)
                f.write("\n")
            print("wrote", path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
