"""The C-ABI library loads without a GPU and exports every symbol declared
in include/mflops_gb300.h; handle creation fails cleanly without a device."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mflops_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mf_\w+)\s*\(", txt, re.M)))


def test_exports_all_declared(mf):
    lib = ctypes.CDLL(mf.lib_path())
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binds_all_declared(mf):
    assert set(declared_symbols()) <= set(mf.exported_symbols())


def test_no_device_is_reported_cleanly(mf):
    import torch
    if torch.cuda.is_available():
        return
    assert mf.device_available() is False
    try:
        mf.DerivativesCoefficients(np.linspace(0, 1, 11), solve=False, so=6)
    except mf.MflopsError as e:
        assert e.code in (mf.MF_ERR_CUDA, mf.MF_ERR_ALLOC)
    else:
        raise AssertionError("handle creation must fail loudly without a GPU")
