"""Writes ref_layout.h: the byte offsets and sizes, in the reference's own
structs GAS, BOX and CELLS (src/cpp_headers.h:145-347), of the fields the
drop-in routines of reference_surface.cpp read and write.

The routines take the reference's struct pointers, so they must address
its fields where its compiler puts them; the numbers are measured here by
compiling a few offsetof() lines against the reference's header (with the
empty MKL stand-ins of oracle/shim), not restated by hand.  Run where the
reference sources are present:

    python monte-carlo-particle-method_gb300/compat/make_layout.py [path/to/reference/src]

(default: $MCPM_REFERENCE_SRC, else the reference checkout beside this
repository).  The header is committed; the drop-in library builds from it
on any host with the same C++ ABI (LP64, libstdc++)."""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_layout.h")

FIELDS = {
    "GAS": ["N", "sigma", "m", "kb", "n", "Fn", "T0", "mu", "visp", "b", "delta_t", "phi", "eqdist", "ast", "bst",
            "crref", "model", "long_range", "Tc", "Th", "n_ratio", "T"],
    "BOX": ["N", "Len", "delta_dim", "direction", "problem", "T_wall_1", "T_wall_2", "T_wall_3", "T_wall_4",
            "U_wall_1", "U_wall_2", "U_wall_3", "U_wall_4", "step", "thermc", "thermh", "file_name"],
    "CELLS": ["num_inside", "indices_inside", "weight", "U_space", "PIJ", "M3", "M4", "M5", "Q", "DM2", "DM4", "Mp",
              "T", "n", "gamma_st", "Lambda", "c", "gamma", "alpha", "beta", "phi", "F2", "omega_max", "crm",
              "divU", "n_smooth", "dn2", "dn3", "n_ratio", "p_m"],
}


def ref_src(argv):
    if len(argv) > 1:
        return argv[1]
    env = os.environ.get("MCPM_REFERENCE_SRC")
    return env or os.path.join(os.path.dirname(REPO), "reference", "src")


HEAD = ("// ref_layout.h -- written by make_layout.py: byte offsets and sizes of the\n"
        "// fields the drop-in routines use in the reference's structs GAS, BOX and\n"
        "// CELLS (src/cpp_headers.h:145-347), measured by compiling offsetof()\n"
        "// against the reference's header.  MCPM_REF_<struct>_<field> is\n"
        "// \"offset, size\" in bytes.  Do not edit: run make_layout.py again.\n"
        "#pragma once\n")


def layout_text(src):
    """The header's text for the reference sources under `src`."""
    if not os.path.isfile(os.path.join(src, "cpp_headers.h")):
        raise FileNotFoundError("reference header not found under %s" % src)
    lines = ['#include "cpp_headers.h"', "#include <cstddef>", "#include <cstdio>", "int main() {"]
    for t, fs in FIELDS.items():
        lines.append('  printf("#define MCPM_REF_SIZEOF_%s %%zu\\n", sizeof(%s));' % (t, t))
        for f in fs:
            lines.append('  printf("#define MCPM_REF_%s_%s %%zu, %%zu\\n", offsetof(%s, %s), sizeof(((%s*)0)->%s));'
                         % (t, f, t, f, t, f))
    lines.append("  return 0;\n}")
    with tempfile.TemporaryDirectory() as d:
        cpp, exe = os.path.join(d, "layout.cpp"), os.path.join(d, "layout")
        with open(cpp, "w") as fh:
            fh.write("\n".join(lines) + "\n")
        shim = os.path.join(REPO, "oracle", "shim")
        subprocess.check_call(["g++", "-std=c++11", "-w", "-I", shim, "-I", src, cpp, "-o", exe])
        body = subprocess.check_output([exe], text=True)
    return HEAD + body


def main(argv):
    try:
        text = layout_text(ref_src(argv))
    except FileNotFoundError as e:
        raise SystemExit(str(e))
    with open(OUT, "w") as fh:
        fh.write(text)
    print(OUT)


if __name__ == "__main__":
    main(sys.argv)
