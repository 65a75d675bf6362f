"""Rewrites CLImage's OpenCL kernel files (demosaic.cl, guided_filter.cl) so that they compile as C++ against cl_shim.h (TEST
INFRASTRUCTURE ONLY).  The output goes to oracle/_ref/ and is never committed.  Only the
syntax C++ lacks is rewritten; no statement of a kernel changes:
  * vector literals (int2)(a, b) / (float4) (v, 0) become constructor calls int2(a, b);
  * the .xyz, .yz and .xy swizzles that are read become calls .xyz() / .yz() / .xy();
  * half literals such as 1.0h become float literals (converted where they are used), and
    every floating constant gets an f suffix (the reference compiles the kernels with
    -cl-single-precision-constant);
  * the file's min / max / abs macros (GNU statement expressions that C++ cannot apply to
    vectors) expand to cl_shim.h's functions instead, the same selects per component;
  * a swizzle that is assigned to (.yz *= s) becomes a write proxy, .yz_ref();
  * x = cond ? a : b; (plain identifiers) becomes clref_select(a, b, cond), which selects
    per component when cond is a vector, as OpenCL does.

    python transform.py <kernels.cl> <out.cpp>
"""
import re
import sys


def transform(src):
    src = re.sub(r"\((int|float|half)([234])\)\s*\(", r"\1\2(", src)
    # a swizzle followed by an assignment operator is written through; elsewhere it is read
    src = re.sub(r"\.(xyz|yz)\b(?=\s*[-+*/]?=(?!=))", r".\1_ref()", src)
    src = re.sub(r"\.xyz\b(?!\s*\(|_ref)", ".xyz()", src)
    src = re.sub(r"\.yz\b(?!\s*\(|_ref)", ".yz()", src)
    src = re.sub(r"\.xy\b(?!\s*\(|_ref|z)", ".xy()", src)
    src = re.sub(r"\b(\d+\.\d*)h\b", r"\1f", src)
    # floating constants are single precision (-cl-single-precision-constant): suffix them
    src = re.sub(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])", r"\1f", src)
    # x = cond ? a : b; with plain identifiers: OpenCL selects per component when cond is a
    # vector, which C++'s ?: cannot do; clref_select does both (a scalar cond picks one side)
    src = re.sub(r"(\b\w+) = ([^;?]+?) \? (\w+) : (\w+);", r"\1 = clref_select(\3, \4, \2);", src)
    # the min / max / abs macros: same names, expanded to the shim's per-component selects
    for name, args in (("min", "a, b"), ("max", "a, b"), ("abs", "a")):
        src = re.sub(r"#define %s\(%s\)(?:[^\n]*\\\n)*[^\n]*\n" % (name, re.escape(args)),
                     "#define %s(%s) clref_%s(%s)\n" % (name, args, name, args), src)
    return src


if __name__ == "__main__":
    with open(sys.argv[1]) as f:
        out = transform(f.read())
    with open(sys.argv[2], "w") as f:
        f.write("// generated from %s by oracle/clref/transform.py; not source of this project\n" % sys.argv[1])
        f.write(out)
