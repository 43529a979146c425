"""Builds the reference-built checker under oracle/_ref/: the reference's own
LBM compute shaders (BoltzmannFluids/Source/GLSL/LBM/*.comp) compiled as C++
on the host, driven by oracle/ref_driver.inc (a restatement of the dispatch
sequence of LBM.cpp).  TEST INFRASTRUCTURE ONLY.

The reference cannot run its shaders here (no graphics stack, GraphicsCortex
not vendored), but the shader sources are C-like.  The recipe lowers them
mechanically -- nothing is rewritten by hand and no source is copied into the
repository; the lowered units are build outputs in oracle/_ref/:

  * drop the two GL-only header lines (shader tag, #version) and the
    compute-shader layout qualifiers;
  * interface blocks become globals: uniform blocks keep their members,
    storage-buffer members `T[] name` become glsl::ssbo<T> (robust access);
  * `uniform` qualifiers go; `T[N] name` array types become std::array;
  * `.xyz` reads become the shim's xyz(), `v.xyz = e` becomes `v = e`;
  * float literals get an f suffix (GLSL literals are single precision);
  * the specialisation macros that GraphicsCortex injects (LBM.cpp:1460-1482)
    are defined per configuration in place of the shader's defaults.

Each configuration in CONFIGS becomes oracle/_ref/libref_<name>.so with the
C API of ref_driver.inc.  Nothing is built when the reference is absent.
"""
import hashlib
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def reference_root(reference=None):
    """The reference checkout: the argument, else the REFERENCE environment
    variable; None when neither names one (nothing is built then)."""
    return reference or os.environ.get("REFERENCE") or None


def shader_dir(root):
    return os.path.join(root, "BoltzmannFluids", "Source", "GLSL", "LBM")

# (namespace, shader file, per-variant macros): collide is compiled three times
# like LBM::_compile_shaders does (LBM.cpp:17-38)
UNITS = [
    ("collide_nosave", "collide", dict(save_macroscopic_variables=0, update_lattices=1)),
    ("collide_save", "collide", dict(save_macroscopic_variables=1, update_lattices=1)),
    ("collide_init", "collide", dict(save_macroscopic_variables=1, update_lattices=0)),
    ("stream", "stream", {}),
    ("stream_thermal", "stream_thermal", {}),
    ("set_equilibrium_populations", "set_equilibrium_populations", {}),
    ("set_equilibrium_populations_thermal", "set_equilibrium_populations_thermal", {}),
]
SHADERS = sorted({u[1] for u in UNITS})
Q_OF = {"D2Q9": 9, "D3Q15": 15, "D3Q19": 19, "D3Q27": 27, "D2Q5": 5, "D3Q7": 7}

# macro names GraphicsCortex injects (LBM.cpp:1460-1482, :17-27)
INJECTED = ["floating_point_accuracy", "velocity_set", "boundry_count", "bits_per_boundry", "periodic_x",
            "periodic_y", "periodic_z", "forcing_scheme", "constant_force", "thermal_flow", "velocity_set_thermal",
            "multiphase_flow", "lattice_is_texutre3d", "lattice_texture3d_internal_format", "esoteric_pull",
            "multiphase_density_texture3d_internal_format", "save_macroscopic_variables", "update_lattices"]

BASE = dict(floating_point_accuracy="fp32", velocity_set="D2Q9", boundry_count=1, bits_per_boundry=0,
            periodic_x=1, periodic_y=1, periodic_z=1, forcing_scheme=0, constant_force=1, thermal_flow=0,
            velocity_set_thermal="D2Q5", multiphase_flow=0, lattice_is_texutre3d=0,
            lattice_texture3d_internal_format="r32f", esoteric_pull=1,
            multiphase_density_texture3d_internal_format="r32f")

# test configurations: name -> macro overrides (matching what the test's inputs make LBM.cpp derive)
CONFIGS = {
    "d2q9_periodic": dict(),
    "d3q19_periodic": dict(velocity_set="D3Q19", velocity_set_thermal="D3Q7"),
    "d3q15_periodic": dict(velocity_set="D3Q15", velocity_set_thermal="D3Q7"),
    "d3q27_periodic": dict(velocity_set="D3Q27", velocity_set_thermal="D3Q7"),
    "d2q9_objects_force": dict(boundry_count=3, bits_per_boundry=2, periodic_x=0, forcing_scheme=1),
    "d2q9_thermal": dict(boundry_count=3, bits_per_boundry=2, periodic_y=0, forcing_scheme=1, thermal_flow=1),
    "d3q19_thermal": dict(velocity_set="D3Q19", velocity_set_thermal="D3Q7", boundry_count=3, bits_per_boundry=2,
                          periodic_y=0, forcing_scheme=1, thermal_flow=1),
    "d2q9_multiphase": dict(multiphase_flow=1),
    "d3q19_multiphase": dict(velocity_set="D3Q19", velocity_set_thermal="D3Q7", multiphase_flow=1),
    "d2q9_two_buffer": dict(boundry_count=3, bits_per_boundry=2, periodic_x=0, periodic_y=0, esoteric_pull=0),
    "d2q9_fp16_texture": dict(floating_point_accuracy="fp16", lattice_is_texutre3d=1,
                              lattice_texture3d_internal_format="r16f"),
    # long runs on the reference's own AA path (skip mode)
    "d2q9_cavity_skip": dict(boundry_count=3, bits_per_boundry=2, periodic_x=0, periodic_y=0, forcing_scheme=1),
    "d3q19_sphere_skip": dict(velocity_set="D3Q19", velocity_set_thermal="D3Q7", boundry_count=2, bits_per_boundry=1),
    "d2q9_von_karman": dict(boundry_count=2, bits_per_boundry=1),
    "d3q19_droplets_limiter": dict(velocity_set="D3Q19", velocity_set_thermal="D3Q7", multiphase_flow=1),
}


def lower(text):
    """Mechanical GLSL -> C++ lowering of one shader (see module docstring)."""
    lines = text.splitlines()
    lines = [l for l in lines if not l.startswith("#<") and not l.startswith("#version")]
    # drop the defaults of injected macros
    out = []
    for l in lines:
        m = re.match(r"\s*#define\s+(\w+)\b", l)
        if m and m.group(1) in INJECTED:
            continue
        out.append(l)
    t = "\n".join(out)
    t = re.sub(r"layout\s*\([^;{]*?\)\s*in\s*;", "", t, flags=re.S)

    def block(m):
        kind, body = m.group(1), m.group(3)
        decls = []
        for d in body.split(";"):
            d = d.strip()
            if not d:
                continue
            a = re.match(r"(\w+)\s*\[\s*\]\s*(\w+)$", d)
            if a:
                decls.append(f"glsl::ssbo<{a.group(1)}> {a.group(2)};")
                continue
            a = re.match(r"(\w+)\s*\[\s*(\w+)\s*\]\s*(\w+)$", d)
            if a:
                decls.append(f"{a.group(1)} {a.group(3)}[{a.group(2)}];")
                continue
            decls.append(d + ";")
        return "\n".join(decls)

    t = re.sub(r"layout\s*\([^)]*\)\s*(uniform|buffer)\s+(\w+)\s*\{(.*?)\}\s*;", block, t, flags=re.S)
    t = re.sub(r"layout\s*\([^)]*\)\s*", "", t)
    t = re.sub(r"\buniform\s+", "", t)
    t = re.sub(r"\b(float|int|uint|vec3|vec4)\[(\w+)\]\s+(\w+)", r"std::array<\1, \2> \3", t)
    t = re.sub(r"(\b\w+)\.xyz\s*=(?!=)", r"\1 =", t)
    t = re.sub(r"\.xyz\b", ".xyz()", t)
    t = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][-+]?\d+)?(?![\w.])", lambda m: m.group(0) + "f", t)
    return t


def velocity_tables(root):
    """The (c, w) tables of VelocitySet.cpp, parsed from the reference's text
    (the same parser that makes tests/golden/velocity_sets.json)."""
    sys.path.insert(0, os.path.join(HERE, "..", "tests", "golden"))
    import make_golden
    text = open(os.path.join(root, "BoltzmannFluids", "Source", "LBMConstants", "VelocitySet.cpp")).read()
    return make_golden.parse_velocity_sets(text)


def unit_source(cfg, tables, root):
    macros = dict(BASE)
    macros.update(cfg)
    parts = ["// generated by oracle/build_ref.py from the reference's shader sources -- do not edit",
             '#include "ref_shim.hpp"']
    for ns, shader, extra in UNITS:
        src = open(os.path.join(shader_dir(root), shader + ".comp")).read()
        low = lower(src)
        defined = sorted(set(re.findall(r"#define\s+(\w+)", src)) | set(INJECTED))
        m = dict(macros)
        m.update(extra)
        for k, v in m.items():
            parts.append(f"#define {k} {v}")
        parts.append(f"namespace ref_{ns} {{")
        parts.append("using namespace glsl;")
        parts.append("uvec3 gl_GlobalInvocationID;")
        parts.append(low)
        parts.append(f"}}  // namespace ref_{ns}")
        for d in defined:
            parts.append(f"#undef {d}")
    q, qt = Q_OF[macros["velocity_set"]], Q_OF[macros["velocity_set_thermal"]]
    cfgs = dict(Q=q, QT=qt, TEX=int(macros["lattice_is_texutre3d"]),
                HALF=int(macros["lattice_texture3d_internal_format"] == "r16f"),
                BOUNDRY_COUNT=macros["boundry_count"], BITS=macros["bits_per_boundry"],
                FORCING=macros["forcing_scheme"], CONSTANT_FORCE=macros["constant_force"],
                THERMAL=macros["thermal_flow"], MULTIPHASE=macros["multiphase_flow"], ESOTERIC=macros["esoteric_pull"])
    for k, v in cfgs.items():
        parts.append(f"#define CFG_{k} {v}")

    def table(name, rows):
        body = ", ".join(f"glsl::vec4({r['c'][0]}, {r['c'][1]}, {r['c'][2]}, (float)({r['w_num']}.0 / {r['w_den']}))"
                         for r in rows)
        return f"static const glsl::vec4 {name}[{len(rows)}] = {{{body}}};"

    parts.append(table("REF_VS", tables[macros["velocity_set"]]))
    parts.append(table("REF_VST", tables[macros["velocity_set_thermal"]]))
    parts.append('#include "ref_driver.inc"')
    return "\n".join(parts) + "\n"


def build(verbose=False, reference=None):
    """Builds every configuration from the reference checkout at `reference`
    (else $REFERENCE); returns {name: path}.  Empty when no checkout is given
    or it lacks the shaders."""
    root = reference_root(reference)
    if not root or not os.path.isdir(shader_dir(root)):
        return {}
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in ("ref_shim.hpp", "ref_driver.inc", "build_ref.py")]
    deps += [os.path.join(shader_dir(root), s + ".comp") for s in SHADERS]
    tables = velocity_tables(root)
    stamp = hashlib.sha1("".join(open(d).read() for d in deps).encode()).hexdigest()[:12]
    built = {}
    procs = []
    for name, cfg in CONFIGS.items():
        so = os.path.join(OUT, f"libref_{name}.so")
        tag = so + ".stamp"
        built[name] = so
        if os.path.exists(so) and os.path.exists(tag) and open(tag).read() == stamp:
            continue
        cpp = os.path.join(OUT, f"ref_{name}.cpp")
        with open(cpp, "w") as f:
            f.write(unit_source(cfg, tables, root))
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
               "-I", HERE, cpp, "-o", so]
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), tag, name))
    for p, tag, name in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"reference build failed for {name}:\n{out[-4000:]}")
        with open(tag, "w") as f:
            f.write(stamp)
        if verbose:
            print("built", name)
    return built


if __name__ == "__main__":
    # python oracle/build_ref.py [reference checkout]  (default: $REFERENCE)
    print(build(verbose=True, reference=sys.argv[1] if len(sys.argv) > 1 else None))
