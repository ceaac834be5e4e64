"""The C-ABI library loads and exports every function that include/*.h
declares (checked without calling into the GPU)."""
import glob
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b((?:sxs|sxsg|point)_?\w*)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_function(lib):
    so = lib.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    decl = declared_functions()
    assert len(decl) > 40
    missing = sorted(decl - exported)
    assert not missing, missing


def test_product_does_not_link_the_oracle(lib):
    out = subprocess.run(["nm", "-D", lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    assert "orc_" not in out and "refh_" not in out
    ldd = subprocess.run(["ldd", lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in ldd
