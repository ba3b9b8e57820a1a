"""Writes the Verner tableau tables (verner_tables.inc) for the device code and the oracle.

The eight Verner pairs of the crate (RKV655e ... RKV989e) are defined by their coefficients, so
the tables hold exactly the crate's values: every decimal literal of
src/tableau/verner.rs is parsed to the nearest double (Python's float(), like Rust's literal
parsing) and written as a hexadecimal float. The stage counts S and I, the order O and the FSAL
flag come from the constructors in src/methods/erk/adaptive/mod.rs.

Usage: python gen_verner_tables.py CRATE_DIR
CRATE_DIR is the root of the crate's source tree (the directory holding src/).  Writes
csrc/verner_tables.inc and oracle/verner_tables.inc.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.normpath(os.path.join(HERE, "..", ".."))
METHODS = ["rkv655e", "rkv656e", "rkv766e", "rkv767e", "rkv877e", "rkv878e", "rkv988e", "rkv989e"]


def constructors(mod_rs):
    """name -> (fsal, O, S, I) from impl_erk_adaptive_step_constructor!(name, fsal, O, S, I, doc)."""
    out = {}
    for m in re.finditer(r"impl_erk_adaptive_step_constructor!\(\s*(\w+),\s*(true|false),\s*(\d+),\s*(\d+),"
                         r"\s*(\d+),", mod_rs):
        out[m.group(1)] = (m.group(2) == "true", int(m.group(3)), int(m.group(4)), int(m.group(5)))
    return out


def parse_block(src, name):
    sig = f"pub fn {name}() -> Self {{"
    start = src.index(sig) + len(sig)
    end = src.index("Self {", start)
    body = src[start:end]
    arrays = {}
    for m in re.finditer(r"let mut (\w+) = \[(\[0\.0; (\d+)\]|0\.0); (\d+)\];", body):
        nm = m.group(1)
        if m.group(3):
            arrays[nm] = [[0.0] * int(m.group(3)) for _ in range(int(m.group(4)))]
        else:
            arrays[nm] = [0.0] * int(m.group(4))
    for m in re.finditer(r"^\s*(\w+)\[(\d+)\](?:\[(\d+)\])?\s*=\s*(-?[0-9][0-9_]*(?:\.[0-9_]*)?(?:e-?[0-9]+)?);",
                         body, re.M):
        nm, i, j, v = m.group(1), int(m.group(2)), m.group(3), float(m.group(4).replace("_", ""))
        if j is None:
            arrays[nm][i] = v
        else:
            arrays[nm][i][int(j)] = v
    bi = [k for k in arrays if k.startswith("bi")]
    assert len(bi) == 1, (name, list(arrays))
    return arrays["c"], arrays["a"], arrays["b"], arrays["bh"], arrays[bi[0]]


def hexf(v):
    return "0.0" if v == 0.0 else v.hex()


def emit(name, spec, tab):
    fsal, order, s, i = spec
    c, a, b, bh, bi = tab
    assert len(c) == i and len(a) == i and len(b) == s and len(bh) == s and len(bi) == i
    row = lambda r: "{" + ", ".join(hexf(x) for x in r) + "}"
    lines = [f"struct {name} {{",
             f"    static constexpr int S = {s}, I = {i}, ORDER = {order};",
             f"    static constexpr bool FSAL = {'true' if fsal else 'false'};",
             f"    static constexpr double C[{i}] = {row(c)};",
             f"    static constexpr double A[{i}][{i}] = {{"]
    lines += [f"        {row(r)}," for r in a]
    lines += ["    };", f"    static constexpr double B[{s}] = {row(b)};",
              f"    static constexpr double BH[{s}] = {row(bh)};",
              f"    static constexpr double BI[{i}][{i}] = {{"]
    lines += [f"        {row(r)}," for r in bi]
    lines += ["    };", "};", ""]
    return "\n".join(lines)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python gen_verner_tables.py CRATE_DIR  (the crate's source tree, holding src/)")
    ref = sys.argv[1]
    src = open(os.path.join(ref, "src", "tableau", "verner.rs")).read()
    specs = constructors(open(os.path.join(ref, "src", "methods", "erk", "adaptive", "mod.rs")).read())
    body = "".join(emit(m, specs[m], parse_block(src, m)) for m in METHODS)
    head = ("// verner_tables.inc — generated by differential-equations_gb300/csrc/gen_verner_tables.py from the\n"
            "// crate's src/tableau/verner.rs (coefficients) and src/methods/erk/adaptive/mod.rs (S, I, O, FSAL).\n"
            "// The methods are defined by these numbers; do not edit by hand.\n"
            "// Layout per method: C[I], A[I][I] (rows S..I-1 are the dense-output stages), B[S], BH[S] (the\n"
            "// embedded lower-order weights), BI[I][I] (BI[i][j]: coefficient of s^(j+1) for stage i).\n")
    for out in (os.path.join(HERE, "verner_tables.inc"), os.path.join(REPO, "oracle", "verner_tables.inc")):
        with open(out, "w") as f:
            f.write(head + "\n" + body)
        print(out)


if __name__ == "__main__":
    main()
