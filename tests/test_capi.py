"""The C-ABI library: it loads, exports every function that include/*.h
declares, and its host-side logic (errors, handles, bundle lookup) behaves
like NCrystal's C interface -- checked without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300._build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b((?:ncrystal|ncgb)_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(B.library_path())
    names = declared_functions(os.path.join(ROOT, "include", "ncrystal_gb300.h"))
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_exports():
    lib = C.CDLL(B.oracle_path())
    for n in ["ncgb_oracle_xs", "ncgb_oracle_xs_many", "ncgb_oracle_scatter", "ncgb_oracle_scatter_many"]:
        assert hasattr(lib, n)


def test_unknown_material_raises_file_not_found():
    with pytest.raises(NC.NCFileNotFound):
        NC.createScatter("NoSuchMaterial_sg1.ncmat;temp=293K")


def test_invalid_handle_sentinels():
    L = NC.lib()
    h = NC.core._Handle(None)
    out = np.zeros(3)
    e = np.ones(3)
    L.ncrystal_crosssection_nonoriented_many(h, e.ctypes.data, 3, 1, out.ctypes.data)
    assert L.ncrystal_error() == 1
    assert L.ncrystal_lasterrortype() == b"LogicError"
    L.ncrystal_clearerror()
    assert np.all(out == -1.0)  # ncrystal.cc:1137-1140
    ef = np.zeros(4)
    mu = np.zeros(4)
    L.ncrystal_samplescatterisotropic_many(h, e.ctypes.data, 2, 2, ef.ctypes.data, mu.ctypes.data)
    L.ncrystal_clearerror()
    assert np.all(ef == -1.0) and np.all(mu == -999.0)  # ncrystal.cc:1237-1244


def test_error_handler_and_halt_default_is_off_in_python():
    L = NC.lib()
    assert L.ncrystal_sethaltonerror(0) == 0  # the Python layer switched halting off
    L.ncrystal_sethaltonerror(0)


def test_halt_on_error_exits_like_reference(tmp_path):
    """Default C behaviour: print the error and exit(1) (ncrystal.cc:296-306)."""
    prog = tmp_path / "halt.c"
    prog.write_text(r'''
#include "ncrystal_gb300.h"
#include <stdio.h>
int main(void){ ncrystal_scatter_t s = ncrystal_create_scatter("NoSuch.ncmat"); (void)s; printf("not reached\n"); return 0; }
''')
    exe = tmp_path / "halt"
    import subprocess
    subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), str(prog), "-o", str(exe),
                           B.library_path(), "-Wl,-rpath," + os.path.dirname(B.library_path())])
    r = subprocess.run([str(exe)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 1
    assert "NCrystal ERROR [FileNotFound]" in r.stdout
    assert "NCrystal terminating due to ERROR" in r.stdout
    assert "not reached" not in r.stdout


def test_bundle_names_match_c_lookup():
    assert B.bundle_file_name(" Al_sg225.ncmat ; temp=293K") == "Al_sg225.ncmat_temp=293K.ncgb"
    assert B.bundle_file_name("X.ncmat;b=1;a=2") == B.bundle_file_name("X.ncmat;a=2;b=1")
