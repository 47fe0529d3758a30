"""The drop-in, built (CPU): PLUTO's own objects without rk_step.o and
split_source.o, linked with pluto-sirocco_gb300/shim/ps_pluto_shim.c and
libps_gb300.so (oracle/ref.mk shim).  The binary must take AdvanceStep and
SplitSource from the shim, and the shim must reach the GPU only through the
C ABI of include/ps_gb300.h.  tests/test_gpu_shim.py runs it."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference():
    import __graft_entry__ as g
    return g.reference_tree()[0]


@pytest.mark.parametrize("cfg", ["blast2d", "wind2d_ode"])
def test_shim_links_into_the_reference_main_loop(built, cfg):
    ref = _reference()
    if not ref:
        pytest.skip("no reference sources here")
    subprocess.run(["make", "-s", "-j8", "-f", os.path.join(ROOT, "oracle", "ref.mk"),
                    "CFG=" + cfg, "REF=" + ref, "shim"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", cfg, "pluto_gb300")
    shim_obj = os.path.join(ROOT, "oracle", "_ref", cfg, "ps_pluto_shim.o")
    defined = subprocess.run(["nm", "--defined-only", shim_obj], capture_output=True,
                             text=True, check=True).stdout
    assert re.search(r" T AdvanceStep$", defined, re.M)
    assert re.search(r" T SplitSource$", defined, re.M)
    # (the reference's own AdvanceStep and SplitSource cannot be in the
    # binary as well: the link would have failed on the duplicate symbols)
    undefined = subprocess.run(["nm", "-u", exe], capture_output=True, text=True,
                               check=True).stdout.split()
    header = open(os.path.join(ROOT, "include", "ps_gb300.h")).read()
    used = sorted({s for s in undefined if s.startswith("ps_")})
    assert "ps_advance_step" in used and "ps_create" in used
    for sym in used:
        assert re.search(r"\b%s\s*\(" % sym, header), sym   # only declared entry points
    if cfg == "wind2d_ode":
        assert "ps_split_source_dt" in used and "ps_set_wind" in used


def test_flux_file_writers_agree(built, tmp_path):
    """The flux files written by liboracle (used for the reference runs of
    the benchmark and the drop-in test) are the ones the golden generator
    wrote in Python for the reference: the same text, byte for byte."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    import ref_runs
    a, b = tmp_path / "c", tmp_path / "py"
    a.mkdir()
    b.mkdir()
    ref_runs.write_wind_flux(str(a), 24, 12, 3.0e37)
    make_golden.write_flux_files(str(b), 24, 12, l_uv=3.0e37)
    for name in ref_runs.FLUX_FILES:
        assert (a / name).read_bytes() == (b / name).read_bytes(), name
