"""The C-ABI library loads and exports every symbol that include/*.h declares
(no compute call: this runs without a GPU)."""
import ctypes
import glob
import os
import re

from conftest import ROOT

# every function the header declares (pic_gpu_*, the ensemble's pic_ens_*, pic_nn_*)
DECL = re.compile(r"^\s*(?:const\s+)?(?:int|char|void|size_t|double|float|unsigned|int64_t|uint32_t|uint64_t)\s*\**\s*"
                  r"(pic_\w+)\s*\(", re.M)


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            names.update(DECL.findall(f.read()))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "pic_gpu_deposit" in names and "pic_gpu_sort" in names and "pic_ens_run" in names and len(names) >= 50


def test_library_exports_every_declared_symbol(pg):
    lib = ctypes.CDLL(pg.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_without_device_are_status_codes(pg):
    # a NULL context is rejected with PIC_ERR_ARG, not a crash
    lib = pg.lib()
    assert lib.pic_gpu_synchronize(None) == -1
    assert b"NULL" in lib.pic_gpu_last_error()


def test_no_cpu_fallback_without_a_device(pg):
    # the product has no CPU path: without a usable GPU, creating a context is an error
    import pytest
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pg.PicError) as e:
        pg.Context(16, 16, 16.0, 16.0, 100)
    assert e.value.code in (-2, -9)  # PIC_ERR_CUDA or PIC_ERR_DEVICE
