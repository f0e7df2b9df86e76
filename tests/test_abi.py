"""CPU checks of the C ABI library: it loads, exports every function the
public header declares, and its host-only pieces agree with the oracle.
No compute call needs a GPU here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(blaze_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import blaze103

    return blaze103.load()


def test_library_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    import blaze103._lib as L

    assert sorted(L.EXPORTS) == sorted(n for n in names if not n.startswith("blaze_noalloc")) or \
        set(L.EXPORTS) <= set(names)


def test_status_strings(lib):
    import blaze103

    assert blaze103.status_string(0) == "ok"
    assert "output" in blaze103.status_string(5)


@pytest.mark.parametrize("qlen,dblen,n", [(300, 7_000_000, 20_000), (1000, 700_000_000, 2_000_000),
                                          (100, 1_800_000_000, 5_000_000), (5000, 180_000_000, 500_000),
                                          (30, 50_000, 200)])
def test_default_params_match_oracle(lib, qlen, dblen, n):
    import blaze103
    import oracle

    p = blaze103.default_params(qlen, db_residues=dblen, db_subjects=n).as_dict()
    o = oracle.default_params(qlen, dblen, n)
    for k in ("word_threshold", "window", "ungapped_xdrop", "ungapped_cutoff", "gap_open",
              "gap_extend", "gapped_xdrop", "gapped_cutoff"):
        assert p[k] == o[k], k
    assert p["eff_searchsp"] == pytest.approx(o["eff_searchsp"], rel=1e-15)
    assert p["lambda"] == o["lam"] and p["K"] == o["K"]
    # published blastp defaults for BLOSUM62 11/1
    assert (p["ungapped_xdrop"], p["gapped_xdrop"], p["word_threshold"], p["window"]) == (16, 38, 11, 40)
    assert p["ungapped_cutoff"] == min(41, p["gapped_cutoff"])


def test_no_device_is_reported_not_faked(lib):
    import blaze103

    if blaze103.device_count() > 0:
        pytest.skip("a GPU is present")
    off = np.array([0, 3], dtype=np.uint64)
    res = np.array([1, 2, 3], dtype=np.uint8)
    h = ctypes.c_void_p()
    st = lib.blaze_db_create(0, res.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                             off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), 1, ctypes.byref(h))
    assert st == 3  # BLAZE_ERR_NO_DEVICE
    with pytest.raises(blaze103.BlazeError):
        blaze103.SeqSrc(res, off)


C_CLIENT = r"""
#include <stdio.h>
#include "blaze_prelim.h"

/* A plain C client of the ABI: the header must compile as C99 and the
 * library link from C. Only calls that need no GPU run here. */
int main(void) {
    blaze_params p;
    int n = 0;
    if (blaze_params_default(300, 7000000ull, 20000u, 10.0, &p) != BLAZE_OK) return 1;
    blaze_device_count(&n);
    printf("%d %d %d %d %d %s\n", p.gapped_cutoff, p.ungapped_cutoff, p.window, p.gapped_xdrop,
           p.hitlist_size, blaze_status_string(BLAZE_ERR_OUTPUT_TOO_SMALL));
    /* every entry point is referenced, so the link checks them all */
    void *fns[] = {(void *)blaze_db_create, (void *)blaze_db_free, (void *)blaze_db_info,
                   (void *)blaze_query_create, (void *)blaze_query_free, (void *)blaze_search_create,
                   (void *)blaze_search_free, (void *)blaze_search_run, (void *)blaze_search_results,
                   (void *)blaze_search_stats, (void *)blaze_search_init_hits, (void *)blaze_prelim_search,
                   (void *)blaze_batch_create, (void *)blaze_batch_free, (void *)blaze_batch_info,
                   (void *)blaze_search_run_batch, (void *)blaze_search_batch_results,
                   (void *)blaze_search_set_tuning, (void *)blaze_search_traceback,
                   (void *)blaze_search_traceback_results, (void *)blaze_search_traceback_batch,
                   (void *)blaze_search_traceback_batch_results, (void *)blaze_server_create,
                   (void *)blaze_server_submit, (void *)blaze_server_wait, (void *)blaze_server_take,
                   (void *)blaze_server_stats_get, (void *)blaze_server_free, (void *)blaze_volume_info,
                   (void *)blaze_volume_read, (void *)blaze_db_open, (void *)blaze_gapped_noalloc,
                   (void *)blaze_last_cuda_error, (void *)blaze_db_create_from_source};
    return fns[0] == 0;
}
"""


def test_header_compiles_and_links_from_c(lib, tmp_path):
    import shutil
    import subprocess

    import blaze103
    import oracle

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    libdir = os.path.dirname(blaze103._lib.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
           "-L", libdir, "-lblaze103", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    o = oracle.default_params(300, 7_000_000, 20_000)
    assert [int(x) for x in out[:5]] == [o["gapped_cutoff"], o["ungapped_cutoff"], 40, 38, 0]
    assert "output" in " ".join(out[5:])


def build_c_client(name: str, out_dir) -> str:
    """Compiles tests/clients/<name>.c as C99 against the public header and
    links it to libblaze103."""
    import shutil
    import subprocess

    import blaze103

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    exe = os.path.join(str(out_dir), name)
    libdir = os.path.dirname(blaze103._lib.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "clients", name + ".c"), "-L", libdir, "-lblaze103",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_seq_source_client_builds_and_reports_no_device(lib, tmp_path):
    import subprocess

    import blaze103

    exe = build_c_client("seqsrc_client", tmp_path)
    if blaze103.device_count() > 0:
        pytest.skip("a GPU is present: tests/test_gpu_seqsrc.py runs the client")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "status 3", r.stdout
