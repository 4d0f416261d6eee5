"""Recipe for the reference-kernel CPU harness (test infrastructure; outputs only into oracle/_ref/).

Steps, all with the host C++ compiler:
  1. compile extract_kernel_text.cpp against the reference sources where they lie
     (<reference>/src/kernel.cpp + kernel.hpp + utilities.hpp) and run it: the output is the
     OpenCL C text the reference JIT-compiles (src/kernel.hpp:7-18);
  2. rewrite the OpenCL vector literals "(float3)(a,b,c)" / "(uint3)(...)" / "(int3)(...)" into
     C++ constructor calls (in C++ the OpenCL form would be a comma expression); nothing else is
     touched;
  3. per variant, write the device defines the reference's host code would inject
     (src/lbm.cpp:334-468; grid size and relaxation rate become runtime variables) and compile
     ref_harness.cpp with -ffp-contract=off into oracle/_ref/ref_<variant>.so.

Where the reference tree is absent (the GPU machine), step 1 is skipped and an already generated
oracle/_ref/gen/kernel_text_cxx.cl is reused if present; the harness is optional everywhere.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
GEN = os.path.join(OUT, "gen")
REFERENCE_SRC = os.environ.get("FX3D_REFERENCE_SRC", "/root/reference/src")
KERNEL_TEXT = os.path.join(GEN, "kernel_text_cxx.cl")

# velocity-set weights as the reference writes them into the kernel defines (src/lbm.cpp:376-394)
_WEIGHTS = {
    19: {"def_w0": "(1.0f/3.0f)", "def_ws": "(1.0f/18.0f)", "def_we": "(1.0f/36.0f)"},
    27: {"def_w0": "(1.0f/3.375f)", "def_ws": "(1.0f/13.5f)", "def_we": "(1.0f/54.0f)", "def_wc": "(1.0f/216.0f)"},
}
_TRANSFERS = {19: 5, 27: 9}


def variant_name(q: int, collision: str, storage: str, extensions: tuple[str, ...] = ()) -> str:
    ext = "".join("_" + e for e in sorted(extensions))
    return f"d3q{q}_{collision}_{storage}{ext}"


def _defines(q: int, collision: str, storage: str, extensions: tuple[str, ...]) -> str:
    lines = [
        "#define def_Nx g_Nx", "#define def_Ny g_Ny", "#define def_Nz g_Nz", "#define def_N g_N",
        "#define uxx uint",
        "#define def_GNx g_Nx", "#define def_GNy g_Ny", "#define def_GNz g_Nz",
        "#define def_Dx 1u", "#define def_Dy 1u", "#define def_Dz 1u",
        "#define def_Ox 0", "#define def_Oy 0", "#define def_Oz 0",
        "#define def_Ax (g_Ny*g_Nz)", "#define def_Ay (g_Nz*g_Nx)", "#define def_Az (g_Nx*g_Ny)",
        f"#define D3Q{q}", f"#define def_velocity_set {q}u", "#define def_dimensions 3u",
        f"#define def_transfers {_TRANSFERS[q]}u",
        "#define def_c 0.57735027f", "#define def_w g_w",
    ]
    lines += [f"#define {k} {v}" for k, v in _WEIGHTS[q].items()]
    lines.append("#define SRT" if collision == "srt" else "#define TRT")
    lines += [
        "#define TYPE_S 0x01", "#define TYPE_E 0x02", "#define TYPE_T 0x04", "#define TYPE_F 0x08",
        "#define TYPE_I 0x10", "#define TYPE_G 0x20", "#define TYPE_X 0x40", "#define TYPE_Y 0x80",
        "#define TYPE_MS 0x03", "#define TYPE_BO 0x03", "#define TYPE_IF 0x18", "#define TYPE_IG 0x30",
        "#define TYPE_GI 0x38", "#define TYPE_SU 0x38", "#define TYPE_XY 0xC0",
    ]
    if storage == "fp16s":
        lines += ["#define fpxx half", "#define fpxx_copy ushort",
                  "#define load(p,o) (vload_half(o,p)*3.0517578E-5f)",
                  "#define store(p,o,x) vstore_half_rte((x)*32768.0f,o,p)"]
    elif storage == "fp16c":
        lines += ["#define fpxx ushort", "#define fpxx_copy ushort",
                  "#define load(p,o) half_to_float_custom((p)[o])",
                  "#define store(p,o,x) (p)[o]=float_to_half_custom(x)"]
    else:
        lines += ["#define fpxx float", "#define fpxx_copy float",
                  "#define load(p,o) (p)[o]", "#define store(p,o,x) (p)[o]=(x)"]
    ext_macro = {"vf": "VOLUME_FORCE", "ff": "FORCE_FIELD", "eq": "EQUILIBRIUM_BOUNDARIES", "sg": "SUBGRID", "mb": "MOVING_BOUNDARIES",
                 "uf": "UPDATE_FIELDS"}
    lines += [f"#define {ext_macro[e]}" for e in extensions]
    return "\n".join(lines) + "\n"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def extract_kernel_text() -> bool:
    """Generate oracle/_ref/gen/kernel_text_cxx.cl; True if available afterwards."""
    os.makedirs(GEN, exist_ok=True)
    kernel_cpp = os.path.join(REFERENCE_SRC, "kernel.cpp")
    if not os.path.isfile(kernel_cpp):
        return os.path.isfile(KERNEL_TEXT)
    exe = os.path.join(OUT, "extract_kernel_text")
    _run(["g++", "-std=c++17", "-O0", "-pthread", "-I", REFERENCE_SRC,
          os.path.join(HERE, "extract_kernel_text.cpp"), "-o", exe])
    text = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    for vec in ("float3", "uint3", "int3"):
        text = text.replace(f"({vec})(", f"{vec}(")
    tmp = KERNEL_TEXT + ".tmp"
    with open(tmp, "w") as f:
        f.write(text)
    os.replace(tmp, KERNEL_TEXT)
    return True


def so_path(name: str) -> str:
    return os.path.join(OUT, f"ref_{name}.so")


def build_variant(q: int, collision: str, storage: str, extensions: tuple[str, ...] = ()) -> str:
    name = variant_name(q, collision, storage, extensions)
    out = so_path(name)
    deps = [KERNEL_TEXT, os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "opencl_c_shim.hpp"),
            os.path.join(ORACLE, "half_ieee.h"), os.path.abspath(__file__)]
    if os.path.isfile(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return out
    defs = os.path.join(GEN, f"defines_{name}.h")
    with open(defs, "w") as f:
        f.write(_defines(q, collision, storage, tuple(extensions)))
    tmp = out + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
          "-w", f'-DREF_DEFINES="{defs}"', f'-DREF_KERNEL_TEXT="{KERNEL_TEXT}"',
          os.path.join(HERE, "ref_harness.cpp"), "-o", tmp])
    os.replace(tmp, out)
    return out


# the variants the parity tests and the CPU baseline use
DEFAULT_VARIANTS = [
    (19, "srt", "fp32", ()),
    (19, "srt", "fp16s", ()),
    (19, "srt", "fp16c", ()),
    (19, "trt", "fp32", ()),
    (19, "trt", "fp16s", ("eq", "ff", "vf")),
    (19, "srt", "fp32", ("eq", "ff", "vf")),
    (19, "trt", "fp32", ("eq", "ff", "vf")),
    (19, "srt", "fp32", ("vf",)),
    (19, "srt", "fp16c", ("eq",)),
    (27, "srt", "fp32", ()),
    (27, "trt", "fp32", ("eq", "ff", "vf")),
    (27, "srt", "fp16s", ()),
    (19, "trt", "fp16s", ("eq",)),
    (19, "trt", "fp32", ("eq",)),
    (19, "srt", "fp32", ("sg",)),
    (19, "trt", "fp16s", ("eq", "sg")),
    (27, "trt", "fp32", ("eq", "ff", "sg", "vf")),
    (19, "srt", "fp32", ("mb",)),
    (19, "trt", "fp16s", ("mb",)),
    (19, "trt", "fp16c", ("mb", "sg")),
    (27, "trt", "fp32", ("eq", "ff", "mb", "vf")),
    (19, "srt", "fp32", ("uf",)),
    (19, "trt", "fp16s", ("eq", "ff", "uf", "vf")),
    (27, "trt", "fp16c", ("eq", "mb", "uf")),
]


def build_all(variants=None, jobs: int | None = None) -> list[str]:
    if not extract_kernel_text():
        return []
    variants = DEFAULT_VARIANTS if variants is None else variants
    jobs = jobs or min(len(variants), os.cpu_count() or 1)
    with ThreadPoolExecutor(jobs) as ex:
        return list(ex.map(lambda v: build_variant(*v), variants))


if __name__ == "__main__":
    built = build_all()
    print("\n".join(built) if built else "reference kernel text unavailable: harness not built")
    sys.exit(0)
