"""The C-ABI library loads and exports every function that
include/fmftsaxs_gb300.h declares, and the libmol2 bridge
(libfmftsaxs_gb300/mol2/sxs_mol2.c, compiled by the caller) defines every
function that include/fmftsaxs_gb300_mol2.h declares (checked without calling
into the GPU)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header, pattern=r"(?:sxs|sxsg|point)_?\w*"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(" + pattern + r")\s*\(", src, flags=re.M):
        names.add(m.group(1))
    return names


def test_library_exports_every_declared_function(lib):
    so = lib.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    decl = declared_functions("fmftsaxs_gb300.h")
    assert len(decl) > 40
    missing = sorted(decl - exported)
    assert not missing, missing


def test_libmol2_bridge_defines_every_declared_function(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler on this host")
    obj = str(tmp_path / "sxs_mol2.o")
    inc = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "tests", "c"), "-I",
           os.path.join(ROOT, "oracle", "shim")]
    subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-c"] + inc +
                   [os.path.join(ROOT, "libfmftsaxs_gb300", "mol2", "sxs_mol2.c"), "-o", obj], check=True)
    out = subprocess.run(["nm", "--defined-only", obj], capture_output=True, text=True, check=True).stdout
    defined = {line.split()[-1] for line in out.splitlines() if " T " in line}
    decl = declared_functions("fmftsaxs_gb300_mol2.h", r"\w+")
    assert {"atom_grp2spf", "atom_grp2spf_inplace", "default_ff_table", "get_ff", "sxs_faccs",
            "sxs_ft_file2euler_file", "mol_atom_group_average_radius"} <= decl
    missing = sorted(decl - defined)
    assert not missing, missing


def test_product_does_not_link_the_oracle(lib):
    out = subprocess.run(["nm", "-D", lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    assert "orc_" not in out and "refh_" not in out
    ldd = subprocess.run(["ldd", lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in ldd
