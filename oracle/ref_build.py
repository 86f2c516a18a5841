"""Builds oracle/_ref/libtrax_ref.so: the reference's own OpenCL kernel text,
compiled for the host CPU.

    python oracle/ref_build.py [--reference PATH]

TEST INFRASTRUCTURE ONLY.  The reference (ThomasHauth/trax) keeps its device
code as OpenCL C inside KERNEL_CLASS / KERNEL_CLASSP macro arguments in its
algorithm headers.  Its host side needs the absent `clever` submodule, Boost,
protobuf 2.4 and an OpenCL runtime, so it cannot be built here; the kernel
text itself needs none of them.  This recipe

  1. reads each kernel of the headers below, where they lie in the reference
     tree, from `__kernel void NAME(` to the end of its body;
  2. removes comments and rewrites the OpenCL vector literals
     `(float3)(a, b, c)` to constructor calls -- the only change to the text;
  3. writes them to oracle/_ref/ref_kernels.inc, one namespace per header;
  4. compiles oracle/ref_host.cpp (the host chain, restated) together with
     that text and oracle/ref_cl.h (the OpenCL built-ins and a work-group
     emulator) into oracle/_ref/libtrax_ref.so with g++ -ffp-contract=off.

Everything it writes goes to oracle/_ref/, which git ignores.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT_DIR, "libtrax_ref.so")
DEFAULT_REFERENCE = os.environ.get("TRAX_REFERENCE_DIR", "/root/reference")

# header (relative to the reference root) -> namespace in ref_kernels.inc
HEADERS = (
    ("src/algorithms/GridBuilder.h", "GridBuilder"),
    ("src/algorithms/PrefixSum.h", "PrefixSum"),
    ("src/algorithms/PairGeneratorBeamspot.h", "PairGeneratorBeamspot"),
    ("src/algorithms/PairGeneratorSector.h", "PairGeneratorSector"),
    ("src/algorithms/TripletThetaPhiPredictor.h", "TripletThetaPhiPredictor"),
    ("src/algorithms/TripletThetaPhiFilter.h", "TripletThetaPhiFilter"),
)

KERNELS = {
    "GridBuilder": ("gridCount", "gridNoLocalCount", "gridStore", "gridWrittenLocalStore",
                    "gridNoLocalStore"),
    "PrefixSum": ("prefixSumWG", "prefixSumPartial", "prefixSumUniformAdd"),
    "PairGeneratorBeamspot": ("pairCount", "pairNoLocalCount", "pairStore"),
    "PairGeneratorSector": ("pairCount", "pairStore"),
    "TripletThetaPhiPredictor": ("predictCount", "predictStore", "predictOffsetMonotonizeStore"),
    "TripletThetaPhiFilter": ("filterCount", "filterPopCount", "filterStore", "filterOffsetStore",
                              "filterOffsetMonotonizeStore"),
}

VECTOR_LITERAL = re.compile(r"\(\s*(float|uint|int)([234])\s*\)\s*\(")


def strip_comments(src: str) -> str:
    """Removes // and /* */ comments, keeping string and character literals
    and every newline (so line numbers still match the header)."""
    out = []
    i, n = 0, len(src)
    while i < n:
        c = src[i]
        if c in "\"'":
            q = c
            j = i + 1
            while j < n and src[j] != q:
                j += 2 if src[j] == "\\" else 1
            out.append(src[i:j + 1])
            i = j + 1
        elif src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("\n" * src.count("\n", i, j))
            i = j
        else:
            out.append(c)
            i += 1
    return "".join(out)


def extract(src: str, name: str):
    """Returns (first line, kernel text) of `__kernel void name(` .. `}`."""
    m = re.search(r"__kernel\s+void\s+" + re.escape(name) + r"\s*\(", src)
    if not m:
        raise SystemExit(f"kernel {name} not found")
    start = m.start()
    depth, j = 0, src.index("{", m.end())
    while True:
        ch = src[j]
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth == 0:
                break
        elif ch in "\"'":
            q = ch
            j += 1
            while src[j] != q:
                j += 2 if src[j] == "\\" else 1
        j += 1
    return src.count("\n", 0, start) + 1, src[start:j + 1]


def generate(reference: str) -> str:
    parts = ["// Generated by oracle/ref_build.py from the reference's kernel text.\n"
             "// Not part of the repository.\n"]
    for rel, ns in HEADERS:
        path = os.path.join(reference, rel)
        with open(path, encoding="utf-8", errors="replace") as f:
            src = strip_comments(f.read())
        parts.append(f"namespace refcl {{ namespace {ns} {{\n")
        for name in KERNELS[ns]:
            line, text = extract(src, name)
            text = VECTOR_LITERAL.sub(lambda m: f"make_{m.group(1)}{m.group(2)}(", text)
            barriers = "true" if re.search(r"\bbarrier\s*\(", text) else "false"
            parts.append(f"// {rel}:{line}\n#line {line} \"{rel}\"\n{text}\n")
            parts.append(f"constexpr bool {name}_barriers = {barriers};\n")
        parts.append("} }\n")
    return "".join(parts)


INC_PATH = os.path.join(OUT_DIR, "ref_kernels.inc")


def build(reference: str = DEFAULT_REFERENCE, verbose: bool = False) -> str:
    """Extracts the kernels when the reference tree is present, then compiles.
    Without the tree an extraction made earlier (oracle/_ref/ref_kernels.inc,
    which travels with the working tree) is compiled as it is."""
    inc = INC_PATH
    if os.path.isdir(os.path.join(reference, "src", "algorithms")):
        os.makedirs(OUT_DIR, exist_ok=True)
        text = generate(reference)
        old = open(inc).read() if os.path.exists(inc) else None
        if old != text:
            with open(inc, "w") as f:
                f.write(text)
    elif not os.path.exists(inc):
        raise FileNotFoundError(f"reference tree not found at {reference} and no earlier "
                                f"extraction in {OUT_DIR}")
    src = os.path.join(HERE, "ref_host.cpp")
    deps = [inc, src, os.path.join(HERE, "ref_cl.h"), os.path.join(HERE, "trax_oracle.h"),
            os.path.join(HERE, "..", "trax_gb300", "csrc", "trax_math.h")]
    if os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d)
                                        for d in deps):
        return LIB_PATH
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++20", "-fPIC", "-shared",
           "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing", "-pthread", "-I", OUT_DIR, "-o", LIB_PATH + ".tmp", src]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    a = ap.parse_args(argv)
    print(build(a.reference, verbose=True))


if __name__ == "__main__":
    sys.exit(main())
