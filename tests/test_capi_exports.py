"""The C-ABI library loads and exports every function include/*.h declares (no GPU calls)."""
import os
import re
import subprocess

import pytest

from radiolensfit2_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("rlf_reference_abi.h", "rlf_gb300.h", "rlf_testing.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            prev = text[max(0, m.start() - 40):m.start()]
            if name in ("if", "for", "while", "return", "sizeof", "defined"):
                continue
            if re.search(r"(double|int|void|char|unsigned int|rlf_observation)\s*\**\s*$", prev):
                names.add(name)
    return names


def test_library_builds_and_loads():
    if not os.path.exists(build.LIB):
        build.build()
    lib = _lib.load()
    assert lib.rlf_version().decode().startswith("rlf-gb300")


def test_every_declared_symbol_is_exported():
    if not os.path.exists(build.LIB):
        build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = declared_functions()
    assert len(declared) >= 35
    missing = sorted(n for n in declared if n not in exported)
    # C++-linkage entry points of marginalise_r.h are exported under their mangled names
    cxx = {"set_posterior_values": "_Z20set_posterior_valuesiPdS_S_S_S_Pi",
           "marginalise_posterior_r": "_Z23marginalise_posterior_riPdS_",
           "marf": "_Z4marfdPv"}
    missing = [n for n in missing if not (n in cxx and cxx[n] in exported)]
    assert missing == []
    for mangled in cxx.values():  # same mangled names as the reference build (marginalise_r.h:24-27)
        assert mangled in exported
    assert set(_lib.EXPORTED) <= exported
