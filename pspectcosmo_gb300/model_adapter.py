"""Compile model.h files written in the reference's model interface into libpsc.so.

The reference changes its physics by editing model.h (model.h:10-104): `num_potential_terms`,
`potential_energy(term, field_values)`, `dvdf(fld, field_values)`, `d2Vdf2(term,
field_values)` and `effective_mass(mass_sq, field_values)`, plus the host-only
`modelinfo_`, `modelinitialize` and `model_output`, all with the helpers of pspectcosmo.h
(`pw2`, `FIELD`, `LOOP`, `DECLARE_INDICES`, `N3`). This module turns such a file, unchanged,
into device code:

* the host-only functions (`modelinfo_`, `modelinitialize`, `model_output`) are dropped;
* every `inline` function becomes `__host__ __device__`;
* `double` becomes the arithmetic type `psc_real`, and every unsuffixed floating literal
  `psc_real(literal)`, so the file compiles twice: once in FP32 (the FP32 lattice path
  evaluates V' in the field precision) and once in FP64;
* `throw ...;` (an invalid term or field index, which the library never passes) becomes
  `__builtin_unreachable();`;
* the lattice-average branch of `potential_energy(term, NULL)` compiles against a `LOOP`
  that runs no iteration: the library calls the model with field values only.

Each listed file becomes user model i (model id PSC_MODEL_USER + i, named by its file
stem) in the generated header `psc_user_models.cuh`, with dispatchers over the ids. The
list comes from the PSC_MODEL_H environment variable (paths separated by os.pathsep) and
defaults to every `.h` file in pspectcosmo_gb300/models/.
"""
from __future__ import annotations

import glob
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
MODELS_DIR = os.path.join(HERE, "models")
MAX_FIELDS = 4
MAX_TERMS = 4
HOST_ONLY = ("modelinfo_", "modelinitialize", "model_output")


def model_paths() -> list[str]:
    env = os.environ.get("PSC_MODEL_H", "").strip()
    if env:
        paths = [os.path.abspath(p) for p in env.split(os.pathsep) if p.strip()]
    else:
        paths = sorted(glob.glob(os.path.join(MODELS_DIR, "*.h")))
    for p in paths:
        if not os.path.isfile(p):
            raise FileNotFoundError(f"model header {p} not found")
    return paths


def model_name(path: str) -> str:
    name = os.path.splitext(os.path.basename(path))[0]
    if not re.fullmatch(r"[A-Za-z_]\w*", name):
        raise ValueError(f"model file name {name!r} is not a C identifier")
    return name


def _strip_comments(text: str) -> str:
    """Remove // and /* */ comments, keeping string and character literals."""
    out, i, n = [], 0, len(text)
    while i < n:
        c = text[i]
        if c in "\"'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            out.append(" ")
            i = n if j < 0 else j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _match_brace(text: str, open_pos: int) -> int:
    """Index one past the brace that closes text[open_pos] == '{'."""
    depth = 0
    i = open_pos
    while i < len(text):
        c = text[i]
        if c in "\"'":
            j = i + 1
            while j < len(text) and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            i = j + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces in model header")


def _drop_function(text: str, name: str) -> str:
    m = re.search(r"(?:\binline\s+)?[\w:<>]+(?:\s*[&*])?\s+\b%s\s*\(" % re.escape(name), text)
    if not m:
        return text
    brace = text.find("{", m.end())
    semi = text.find(";", m.end())
    if brace < 0 or (0 <= semi < brace):   # a declaration only
        return text[:m.start()] + text[semi + 1:]
    return text[:m.start()] + text[_match_brace(text, brace):]


_FLOAT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def process(text: str) -> str:
    """model.h text -> the body compiled once per arithmetic type (see the module doc)."""
    text = _strip_comments(text)
    text = "\n".join(ln for ln in text.splitlines() if not re.match(r"\s*#\s*include\b", ln))
    for name in HOST_ONLY:
        text = _drop_function(text, name)
    text = re.sub(r"\bthrow\b[^;]*;", "__builtin_unreachable();", text)
    text = re.sub(r"\bdouble\b", "psc_real", text)
    text = _FLOAT.sub(lambda m: "psc_real(%s)" % m.group(1), text)
    text = re.sub(r"\binline\b", "__host__ __device__ inline", text)
    return text


def generate(paths: list[str] | None = None) -> str:
    paths = model_paths() if paths is None else paths
    names = [model_name(p) for p in paths]
    if len(set(names)) != len(names):
        raise ValueError(f"duplicate model names in {names}")
    out = [
        "// psc_user_models.cuh: GENERATED by pspectcosmo_gb300/model_adapter.py from",
        *[f"//   {p}" for p in paths],
        "// Each model.h compiles twice, in FP32 (namespace um_<name>_f32) and FP64 (um_<name>_f64).",
        "#pragma once",
        "#include <cmath>",
        "#include <cstddef>",
        "#include <cstdlib>",
        "#include <stdexcept>",
        "#ifndef __CUDACC__",
        "#ifndef __host__",
        "#define __host__",
        "#endif",
        "#ifndef __device__",
        "#define __device__",
        "#endif",
        "#endif",
        "namespace psc {",
        "#define DECLARE_INDICES",
        "#define LOOP for (int psc_um_never_ = 0; psc_um_never_ < 0; ++psc_um_never_)",
        "#define FIELD(fld) psc_real(0)",
        "#define N3 psc_real(1)",
    ]
    for p, name in zip(paths, names):
        with open(p) as fh:
            body = process(fh.read())
        for suffix, real in (("f32", "float"), ("f64", "double")):
            out += [
                f"namespace um_{name}_{suffix} {{",
                f"typedef {real} psc_real;",
                "__host__ __device__ inline psc_real pw2(psc_real x) { return x * x; }",
                body,
                f"}}  // namespace um_{name}_{suffix}",
            ]
    out += ["#undef DECLARE_INDICES", "#undef LOOP", "#undef FIELD", "#undef N3", ""]
    n = len(names)
    out.append(f"constexpr int kUserModels = {n};")
    out.append(f"constexpr int kUserMaxFields = {MAX_FIELDS};")
    out.append(f"constexpr int kUserMaxTerms = {MAX_TERMS};")
    out.append("static const char *const kUserModelNames[%d] = {%s};" % (max(n, 1), ", ".join(
        f'"{nm}"' for nm in names) if n else '""'))
    for name in names:
        out.append(f"static_assert(um_{name}_f64::num_potential_terms >= 1 && um_{name}_f64::num_potential_terms <= "
                   f"{MAX_TERMS}, \"model {name}: num_potential_terms must be 1..{MAX_TERMS}\");")
    out.append("__host__ __device__ inline int um_nterms(int i) {")
    out.append("    switch (i) {")
    for i, name in enumerate(names):
        out.append(f"    case {i}: return um_{name}_f64::num_potential_terms;")
    out.append("    default: return 0;\n    }\n}")
    # dispatchers: T selects the FP32 or FP64 compilation of each model
    for fn, sig, call in (
        ("um_dvdf", "const T *v, T *out, int nf",
         "for (int q = 0; q < nf; ++q) out[q] = NS::dvdf(q, v);"),
        ("um_potential", "const T *v, T *terms",
         "for (int t = 0; t < NS::num_potential_terms; ++t) terms[t] = NS::potential_energy(t, const_cast<T *>(v));"),
        ("um_effective_mass", "const T *v, T *m2",
         "NS::effective_mass(m2, const_cast<T *>(v));"),
    ):
        out.append(f"template <typename T> __host__ __device__ inline void {fn}(int i, {sig}) {{")
        out.append("    switch (i) {")
        for i, name in enumerate(names):
            out.append(f"    case {i}: {{")
            out.append(f"        if constexpr (sizeof(T) == 4) {{ namespace NS = um_{name}_f32; {call} }}")
            out.append(f"        else {{ namespace NS = um_{name}_f64; {call} }}")
            out.append("        break;\n    }")
        out.append("    default: break;\n    }\n}")
    out.append("}  // namespace psc")
    return "\n".join(out) + "\n"


def write(path: str, paths: list[str] | None = None) -> bool:
    """Write the generated header; returns True when its content changed."""
    text = generate(paths)
    old = None
    if os.path.exists(path):
        with open(path) as fh:
            old = fh.read()
    if old == text:
        return False
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as fh:
        fh.write(text)
    return True
