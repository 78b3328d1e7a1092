"""OpenCL C -> C++ translation of the reference's kernel strings (oracle harness only).

The reference compiles its device code at run time from OpenCL C source strings
(``prg = Program(ctx, r\"\"\" ... \"\"\")`` at radon_tgv_primal_dual_3d.py:96-848 and
radon_tgv_primal_dual_2d.py:95-463).  No OpenCL platform exists here, so the
stand-in ``pyopencl`` of this package hands each such string to :func:`translate`,
which rewrites it into C++ over ``oclcpp.h`` and adds one OpenMP launcher per
``__kernel`` that walks the 3-D NDRange.  The kernel bodies are not edited beyond
the mechanical syntax mapping below, so the arithmetic that runs is the
reference's own.

Mapping:
  (floatN)(args)         -> make_vN(args)
  v.sK / v.SK / v.x..w   -> v.c[K]
  v.sKLM                 -> v.sw<K,L,M>()
  float* helpers returning a local array -> that array made ``static thread_local``
    (the original returns a dangling pointer, radon_tgv_primal_dual_3d.py:219-220,
    282-283; this gives it the defined meaning the callers rely on).
  Kernels that never read get_global_id(2) but are launched with a third extent
  > 1 (the 2-D Frobenius/nuclear projections, radon_tgv_primal_dual_2d.py:643-648)
  run once per (x, y): all copies would compute the same idempotent update, and
  running them concurrently on a GPU is one of the schedules this reproduces.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

_COMP = {"x": 0, "y": 1, "z": 2, "w": 3}


@dataclass
class Param:
    ctype: str
    name: str
    pointer: bool


@dataclass
class KernelSig:
    name: str
    params: list = field(default_factory=list)
    uses_z: bool = True


def _parse_params(text: str) -> list:
    out = []
    text = text.strip()
    if not text:
        return out
    for raw in text.split(","):
        t = raw.replace("__global", " ").replace("__constant", " ").replace("const", " ")
        pointer = "*" in t
        t = t.replace("*", " ")
        toks = t.split()
        out.append(Param(ctype=toks[0], name=toks[1], pointer=pointer))
    return out


def _kernel_bodies(src: str):
    """Yield (name, params_text, body_text) for every __kernel in ``src``."""
    for m in re.finditer(r"__kernel\s+void\s+(\w+)\s*\(([^)]*)\)\s*\{", src):
        depth, i = 1, m.end()
        while depth:
            ch = src[i]
            depth += (ch == "{") - (ch == "}")
            i += 1
        yield m.group(1), m.group(2), src[m.end():i - 1]


def extract_kernel_source(py_text: str) -> str:
    """Return the OpenCL C string passed to ``Program(ctx, r\"\"\"...\"\"\")``."""
    m = re.search(r'Program\(\s*ctx\s*,\s*r"""(.*?)"""\s*\)', py_text, re.S)
    if not m:
        raise ValueError("no Program(ctx, r\"\"\"...\"\"\") kernel string found")
    return m.group(1)


def _swizzle(m: re.Match) -> str:
    digits = m.group(2)
    idx = [int(d, 16) for d in digits]
    if len(idx) == 1:
        return f".c[{idx[0]}]"
    return ".sw<" + ",".join(str(k) for k in idx) + ">()"


def _static_local_arrays(body: str) -> str:
    # float name[K] = {a, b, ...};   ->  static thread_local storage, re-filled every call
    def rep(m):
        name, k, init = m.group(1), m.group(2), m.group(3)
        return (f"static thread_local float {name}[{k}]; "
                f"{{ float __t[{k}] = {{{init}}}; for (int __q = 0; __q < {k}; ++__q) {name}[__q] = __t[__q]; }}")
    return re.sub(r"\bfloat\s+(\w+)\s*\[(\d+)\]\s*=\s*\{([^}]*)\}\s*;", rep, body)


def translate(cl_src: str) -> tuple[str, list]:
    """Translate an OpenCL C program into (C++ source, [KernelSig])."""
    sigs = []
    for name, ptxt, body in _kernel_bodies(cl_src):
        sigs.append(KernelSig(name=name, params=_parse_params(ptxt), uses_z="get_global_id(2)" in body))

    s = cl_src
    s = re.sub(r"\(\s*float([2348])\s*\)\s*\(", r"make_v\1(", s)
    s = re.sub(r"\.([sS])([0-9a-fA-F]+)\b", _swizzle, s)
    s = re.sub(r"\.([xyzw])\b", lambda m: f".c[{_COMP[m.group(1)]}]", s)
    s = _static_local_arrays(s)
    s = re.sub(r"__kernel\s+", "", s)
    s = re.sub(r"\b__global\b|\b__constant\b", "", s)

    lines = ['#include "oclcpp.h"', "namespace ocl {",
             "thread_local size_t g_gid[3];", "thread_local size_t g_gsz[3];", s, "}  // namespace ocl", ""]
    for sig in sigs:
        args = []
        for k, p in enumerate(sig.params):
            t = f"ocl::{p.ctype}" if p.ctype.startswith("float") and p.ctype != "float" else p.ctype
            args.append(f"({t}*)args[{k}]" if p.pointer else f"*({t}*)args[{k}]")
        call = f"ocl::{sig.name}({', '.join(args)});"
        zext = "g2" if sig.uses_z else "(size_t)1"
        lines.append(f'extern "C" void launch_{sig.name}(size_t g0, size_t g1, size_t g2, void **args) {{')
        lines.append("  (void)args;")
        lines.append(f"  const size_t gz = {zext};")
        lines.append("#pragma omp parallel for collapse(2) schedule(static)")
        lines.append("  for (size_t z = 0; z < gz; ++z)")
        lines.append("    for (size_t y = 0; y < g1; ++y) {")
        lines.append("      ocl::g_gsz[0] = g0; ocl::g_gsz[1] = g1; ocl::g_gsz[2] = g2;")
        lines.append("      ocl::g_gid[1] = y; ocl::g_gid[2] = z;")
        lines.append(f"      for (size_t x = 0; x < g0; ++x) {{ ocl::g_gid[0] = x; {call} }}")
        lines.append("    }")
        lines.append("}")
    return "\n".join(lines) + "\n", sigs


def translate_elementwise(arguments: str, operation: str) -> str:
    """C++ for pyopencl's ElementwiseKernel(ctx, arguments, operation)."""
    decls = []
    for k, a in enumerate(arguments.split(",")):
        t = a.strip()
        ctype, name = t.replace("*", " * ").split()[0], t.replace("*", " ").split()[-1]
        decls.append(f"  {ctype} *{name} = ({ctype}*)args[{k}];")
    return "\n".join([
        "#include <cstddef>",
        'extern "C" void launch_elementwise(size_t n, void **args) {',
        *decls,
        "#pragma omp parallel for schedule(static)",
        "  for (size_t i = 0; i < n; ++i) {", f"    {operation};", "  }", "}", ""])
