"""The C-ABI library loads and exports every symbol declared in include/*.h
(no compute calls: this runs without a GPU)."""
import glob
import os
import re
import subprocess

import pytest

from conftest import REFERENCE, ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.add(name)
    return names


def test_library_exports_every_declared_symbol(lib):
    from asd_pocs_mex_cuda_demo_gb300._lib import LIB_PATH

    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    declared = _declared()
    assert "Ax_cone_mf_gpu_new" in declared and "asdpocs_plan_run" in declared
    missing = sorted(declared - exported)
    assert not missing, missing
    for name in declared:
        getattr(lib, name)  # resolvable through ctypes


def test_python_signatures_cover_header():
    from asd_pocs_mex_cuda_demo_gb300._lib import SIGNATURES

    bound = {s[0] for s in SIGNATURES}
    assert _declared() == bound


def test_version_and_error_state_without_gpu(lib):
    assert b"sm_103a" in lib.asdpocs_version()
    # a refused call sets the calling thread's status and message; the next
    # successful call clears them
    assert lib.asdpocs_store_sinogram(None, None, 4, 0) == 1
    assert lib.asdpocs_last_status() == 1 and b"null" in lib.asdpocs_last_error()
    assert lib.asdpocs_store_sinogram(None, None, 0, 0) == 0
    assert lib.asdpocs_last_status() == 0


def test_launcher_signatures_match_reference_arity():
    # Ax_cone_gpu.cu:778-779 (16 args) and :299-300 (18 args)
    from asd_pocs_mex_cuda_demo_gb300._lib import SIGNATURES

    sig = {s[0]: s[2] for s in SIGNATURES}
    assert len(sig["Ax_cone_mf_gpu_new"]) == 16
    assert len(sig["Atx_cone_mf_gpu_new"]) == 18


def test_ref_signatures_in_reference_source_if_present():
    ref = os.path.join(REFERENCE, "src", "AxAtx", "Ax_cone_gpu.cu")
    if not os.path.exists(ref):
        pytest.skip("reference checkout not on this machine")
    src = open(ref, encoding="latin-1").read()
    hdr = open(os.path.join(ROOT, "include", "asdpocs_gb300.h")).read()

    def params(text, name):
        m = re.search(r'extern\s+"C"\s+void\s+' + name + r"\s*\(([^)]*)\)", text)
        if m is None:
            m = re.search(r"void\s+" + name + r"\s*\(([^)]*)\)", text)
        return [p.split()[-1].strip("*") for p in m.group(1).replace("\n", " ").split(",")]

    for name in ("Ax_cone_mf_gpu_new", "Atx_cone_mf_gpu_new"):
        assert params(src, name) == params(hdr, name), name


def test_normal_build_has_no_bounds_checks(lib):
    """asdpocs_checked_errors exists in every build; only the bounds-checked
    variant (libasdpocs_gb300_checked.so) counts, the normal one refuses."""
    import ctypes as C

    from asd_pocs_mex_cuda_demo_gb300._lib import AsdpocsError, check

    cnt, first = C.c_ulonglong(), (C.c_longlong * 2)()
    with pytest.raises(AsdpocsError, match="not a bounds-checked build"):
        check(lib.asdpocs_checked_errors(C.byref(cnt), first))
