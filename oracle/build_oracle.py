"""Build recipe for the oracle (test infrastructure only).

Builds
  oracle/liboz_oracle.so        -- the CPU restatement (oz_oracle.c), gcc + OpenMP
  oracle/_ref/libref_decode.so  -- the reference's own convert_paired_i64_to_double_matrix
                                   (include/oz_aie.h:92-150), only when the reference
                                   sources are present at REFERENCE_ROOT: the
                                   environment variable OZAIE_REFERENCE_ROOT, else a
                                   checkout named "reference" beside this repository.

Outputs go only to oracle/ and oracle/_ref/ (both git-ignored binaries).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get("OZAIE_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
ORACLE_SO = os.path.join(HERE, "liboz_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libref_decode.so")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force=False):
    src = os.path.join(HERE, "oz_oracle.c")
    hdr = os.path.join(HERE, "oz_oracle.h")
    if not force and _newer(ORACLE_SO, [src, hdr]):
        return ORACLE_SO
    cmd = ["gcc", "-O3", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wno-unused-function",
           src, "-o", ORACLE_SO, "-ldl", "-lm"]
    subprocess.check_call(cmd)
    return ORACLE_SO


def _extract_function(text, name):
    """Return the full definition of C++ function `name` (signature through the
    matching closing brace) from `text`."""
    m = re.search(r"void\s+" + re.escape(name) + r"\s*\(", text)
    if not m:
        raise RuntimeError("function %s not found in reference header" % name)
    i = text.index("{", m.end())
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[m.start():j + 1]
    raise RuntimeError("unbalanced braces while extracting %s" % name)


def build_ref_decode(force=False):
    """Compile the reference's decode from its own header; None if absent."""
    header = os.path.join(REFERENCE_ROOT, "include", "oz_aie.h")
    if not os.path.exists(header):
        return None
    shim = os.path.join(HERE, "ref_decode_shim.cpp")
    if not force and _newer(REF_SO, [header, shim]):
        return REF_SO
    os.makedirs(REF_DIR, exist_ok=True)
    with open(header) as f:
        body = _extract_function(f.read(), "convert_paired_i64_to_double_matrix")
    with open(os.path.join(REF_DIR, "ref_decode_body.inc"), "w") as f:
        f.write("// extracted at build time from %s\n" % header)
        f.write(body + "\n")
    cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-I", HERE, shim, "-o", REF_SO]
    subprocess.check_call(cmd)
    return REF_SO


def build_all(force=False):
    out = {"oracle": build_oracle(force)}
    out["ref_decode"] = build_ref_decode(force)
    return out


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
