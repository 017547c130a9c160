"""Build recipe for ``oracle/_ref``: the reference's OWN CPU fluid functions, compiled here.

Test infrastructure only.  The reference tree cannot be built as shipped (its
``rx_utility.h`` is missing, and its headers pull in GLUT/FLTK/boost), but the
CPU fluid path itself is plain C++.  This script reads the reference sources
where they lie, cuts out -- by signature anchor plus brace matching, never by
hand -- exactly the functions on the fluid path, and writes them into the
git-ignored ``oracle/_ref/src/`` next to this project's own shim headers
(``shim/rx_utility.h``) and harness classes (``harness_classes.h``,
``harness_api.cpp``).  ``build_ref()`` then compiles that translation unit into
``oracle/_ref/libfsph_ref.so``.

Functions taken (reference file:line of each anchor):
  rx_kernel.h             whole file (kernel functions and coefficients)
  rx_nnsearch.h:39-65     rxHashSort, LessHash, rxNeigh
  rx_nnsearch.h:70        class rxNNGrid (declaration only)
  rx_nnsearch.h:174,225   rxNNGrid::Setup, rxNNGrid::SetObjectToCell
  rx_nnsearch.h:454,487   rxNNGrid::GetNN, rxNNGrid::getNeighborsInCell
  rx_nnsearch.h:578,590   rxNNGrid::CalGridHash (both overloads)
  rx_sph_solid.h:29       class rxCollisionInfo
  rx_sph.h:95             struct rxSPHEnviroment
  rx_sph_solid.cpp:23,44  RX_AABB_NORMALS, AABB_point_dist
  rx_sph_solid.cpp:244    rxSolidBox::GetDistanceR
  rx_sph_pbd.cpp:102-1747 rxPBDSPH::{Initialize, Update, calDensity, calForceExtAndVisc,
                          calScalingFactor, calPositionCorrection, calRestDensity,
                          calCollisionSolid, integrate, GetNearestNeighbors, SetParticlesToCell}
  rx_sph_cpu.cpp:92-1377  rxSPH::{Initialize, Update, calDensity, calForce, calRestDensity,
                          calCollisionSolid, integrate, GetNearestNeighbors, SetParticlesToCell}

The generated sources are never committed (``oracle/_ref/`` is git-ignored);
when the reference tree is absent (the GPU host) an already-extracted
``oracle/_ref/src`` is compiled as is, and if there is none the reference pin
is reported as unavailable.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REF_OUT = os.path.join(ORACLE, "_ref")
SRC_OUT = os.path.join(REF_OUT, "src")
# The reference checkout: $FSPH_REFERENCE_ROOT, else a sibling directory
# "reference" beside this repository.
REF_ROOT = os.environ.get("FSPH_REFERENCE_ROOT") or os.path.normpath(
    os.path.join(ORACLE, "..", "..", "reference"))


def _read(name: str) -> list[str]:
    with open(os.path.join(REF_ROOT, name), "rb") as f:
        return f.read().decode("cp932").replace("\r\n", "\n").split("\n")


def _block(lines: list[str], anchor: str, *, nth: int = 0, until_semicolon: bool = False) -> str:
    """Return the text from the line matching ``anchor`` (regex, at line start) to
    the brace that closes its first ``{`` (plus the trailing ``;`` for a type)."""
    rx = re.compile(anchor)
    hits = [i for i, l in enumerate(lines) if rx.match(l)]
    if len(hits) <= nth:
        raise RuntimeError(f"anchor not found: {anchor!r}")
    start = hits[nth]
    depth = 0
    opened = False
    out = []
    for i in range(start, len(lines)):
        line = lines[i]
        code = line.split("//")[0]
        out.append(line)
        for ch in code:
            if ch == "{":
                depth += 1
                opened = True
            elif ch == "}":
                depth -= 1
        if opened and depth == 0:
            if until_semicolon and ";" not in code[code.rfind("}"):]:
                # type declaration: keep going to the terminating ';'
                j = i + 1
                while ";" not in lines[j]:
                    out.append(lines[j])
                    j += 1
                out.append(lines[j])
            break
    else:
        raise RuntimeError(f"unbalanced braces after {anchor!r}")
    return f"#line {start + 1}\n" + "\n".join(out) + "\n"


def _statement(lines: list[str], anchor: str) -> str:
    rx = re.compile(anchor)
    for i, l in enumerate(lines):
        if rx.match(l):
            out = []
            j = i
            while True:
                out.append(lines[j])
                if ";" in lines[j].split("//")[0]:
                    break
                j += 1
            return f"#line {i + 1}\n" + "\n".join(out) + "\n"
    raise RuntimeError(f"anchor not found: {anchor!r}")


def extract() -> bool:
    """Write oracle/_ref/src/*.  Returns False when the reference tree is absent."""
    if not os.path.isfile(os.path.join(REF_ROOT, "rx_sph_pbd.cpp")):
        return False
    os.makedirs(SRC_OUT, exist_ok=True)

    kern = _read("rx_kernel.h")
    with open(os.path.join(SRC_OUT, "rx_kernel.h"), "w") as f:
        f.write("\n".join(kern))

    nn = _read("rx_nnsearch.h")
    solid_h = _read("rx_sph_solid.h")
    solid = _read("rx_sph_solid.cpp")
    sph_h = _read("rx_sph.h")
    pbd = _read("rx_sph_pbd.cpp")
    cpu = _read("rx_sph_cpu.cpp")

    parts = []
    parts.append('#line 1 "rx_nnsearch.h"\n')
    parts.append(_block(nn, r"^struct rxHashSort", until_semicolon=True))
    parts.append(_block(nn, r"^inline bool LessHash"))
    parts.append(_block(nn, r"^struct rxNeigh", until_semicolon=True))
    parts.append(_block(nn, r"^class rxNNGrid", until_semicolon=True))
    parts.append("#define cout fsph_ref_null_stream\n")
    parts.append(_block(nn, r"^inline void rxNNGrid::Setup"))
    parts.append("#undef cout\n")
    parts.append(_block(nn, r"^inline void rxNNGrid::SetObjectToCell"))
    parts.append(_block(nn, r"^inline void rxNNGrid::GetNN\("))
    parts.append(_block(nn, r"^inline void rxNNGrid::getNeighborsInCell"))
    parts.append(_block(nn, r"^inline uint rxNNGrid::CalGridHash\(int"))
    parts.append(_block(nn, r"^inline uint rxNNGrid::CalGridHash\(Vec3"))
    parts.append('#line 1 "rx_sph_solid.h"\n')
    parts.append(_block(solid_h, r"^class rxCollisionInfo", until_semicolon=True))
    parts.append('#line 1 "rx_sph.h"\n')
    parts.append(_block(sph_h, r"^struct rxSPHEnviroment", until_semicolon=True))
    with open(os.path.join(SRC_OUT, "ref_types.inc"), "w") as f:
        f.write("".join(parts))

    parts = ['#line 1 "rx_sph_solid.cpp"\n']
    parts.append(_statement(solid, r"^const Vec3 RX_AABB_NORMALS"))
    parts.append(_block(solid, r"^bool AABB_point_dist"))
    parts.append(_block(solid, r"^bool rxSolidBox::GetDistanceR"))
    parts.append('#line 1 "rx_sph_pbd.cpp"\n')
    for a in [r"^void rxPBDSPH::Initialize", r"^bool rxPBDSPH::Update", r"^void rxPBDSPH::calDensity",
              r"^void rxPBDSPH::calForceExtAndVisc", r"^void rxPBDSPH::calScalingFactor",
              r"^void rxPBDSPH::calPositionCorrection", r"^RXREAL rxPBDSPH::calRestDensity",
              r"^int rxPBDSPH::calCollisionSolid", r"^void rxPBDSPH::integrate",
              r"^void rxPBDSPH::GetNearestNeighbors\(int", r"^void rxPBDSPH::GetNearestNeighbors\(Vec3",
              r"^void rxPBDSPH::SetParticlesToCell\(RXREAL", r"^void rxPBDSPH::SetParticlesToCell\(void",
              r"^double rxPBDSPH::GetImplicit", r"^void rxPBDSPH::CalImplicitField\(", r"^double rxPBDSPH::CalColorField"]:
        parts.append(_block(pbd, a))
    parts.append('#line 1 "rx_sph_cpu.cpp"\n')
    for a in [r"^void rxSPH::Initialize", r"^bool rxSPH::Update", r"^void rxSPH::calDensity",
              r"^void rxSPH::calForce\(", r"^RXREAL rxSPH::calRestDensity",
              r"^int rxSPH::calCollisionSolid", r"^void rxSPH::integrate",
              r"^void rxSPH::GetNearestNeighbors\(int", r"^void rxSPH::GetNearestNeighbors\(Vec3",
              r"^void rxSPH::SetParticlesToCell\(RXREAL", r"^void rxSPH::SetParticlesToCell\(void"]:
        parts.append(_block(cpu, a))
    with open(os.path.join(SRC_OUT, "ref_funcs.inc"), "w") as f:
        f.write("".join(parts))

    with open(os.path.join(SRC_OUT, "ref_tu.cpp"), "w") as f:
        f.write('// generated by oracle/ref_harness/extract.py -- do not edit, do not commit\n'
                '#include "harness_prelude.h"\n'
                '#include "rx_kernel.h"\n'
                '#include "ref_types.inc"\n'
                '#include "harness_classes.h"\n'
                '#include "ref_funcs.inc"\n'
                '#include "harness_api.cpp"\n')
    return True


def build_ref(verbose: bool = False) -> str | None:
    """Extract (when the reference tree is present) and compile oracle/_ref/libfsph_ref.so.

    Returns the library path, or None when neither the reference tree nor an
    extracted copy is available."""
    have = extract()
    tu = os.path.join(SRC_OUT, "ref_tu.cpp")
    if not have and not os.path.isfile(tu):
        return None
    out = os.path.join(REF_OUT, "libfsph_ref.so")
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
           "-I", SRC_OUT, "-I", os.path.join(HERE, "shim"), "-I", HERE,
           "-w", tu, "-o", out]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    p = build_ref(verbose=True)
    print(p if p else "reference sources unavailable")
    sys.exit(0)
