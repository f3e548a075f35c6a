"""The C-ABI library loads without a GPU and exports every function the
public headers declare (no compute calls here)."""
import ctypes
import os
import subprocess

import ltpmg_gb300 as G


def test_library_exports_every_declared_symbol(lib):
    names = G.header_functions()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", G.lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_status_strings(lib):
    for s in range(-7, 1):
        assert lib.ltp_status_string(s)
    assert lib.ltp_version().startswith(b"ltpmg_gb300")


def test_init_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        return
    cfg = G.lib.Config(0, 0, 0, 0, 0)
    h = ctypes.c_void_p()
    rc = lib.ltp_init(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == G.lib.LTP_E_CUDA and not h.value


def test_null_arguments_rejected(lib):
    assert lib.ltp_init(None, None) == G.lib.LTP_E_BADARG
    assert lib.ltp_shutdown(None) == G.lib.LTP_E_BADARG
    assert lib.ltp_batch_free(None, None) == G.lib.LTP_E_BADARG


def test_pinned_alloc_without_gpu_is_null_or_valid(lib):
    p = lib.ltp_host_alloc(64)
    if p:
        lib.ltp_host_free(p)


def test_build_artifacts_in_tree():
    assert os.path.dirname(G.lib.LIB_PATH).endswith("ltpmg_gb300")


def test_binding_constants_match_the_header():
    """The ctypes binding's flag, mode, rule, op and status constants equal
    the header's #defines."""
    import re

    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "ltpmg_gb300.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define LTP_(\w+)\s+\(?(-?\d+)u?\)?", hdr)}
    for name in ("SERVE_EAGER", "SERVE_KEEP_RESULTS", "SERVE_PERSISTENT", "SERVE_KEYS64", "SERVE_JIT",
                 "SERVE_MAX_OPS", "MODE_STREAM", "MODE_GRAPH", "MODE_PERSISTENT", "RULE_ORDERED", "RULE_PRIORITY",
                 "OP_READ", "OP_ADD", "OP_INSERT", "FLAG_STAGE_TIMING", "TUNE_MARK_PRECHECK"):
        assert name in defs, name
        assert getattr(G.lib, name) == defs[name], name
    for name in ("E_BADARG", "E_CUDA", "E_CAPACITY", "E_TIMEOUT", "E_DEVICE_ASSERT", "E_NOMEM", "E_STATE"):
        assert getattr(G.lib, "LTP_" + name) == defs[name], name


def test_probe_is_outside_the_product_library():
    """The benchmark's random-access probe builds into its own library; the
    product library exports no probe."""
    out = subprocess.run(["nm", "-D", "--defined-only", G.lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "ltp_probe_random_access" not in out
    assert os.path.exists(G.lib.PROBE_LIB_PATH)
    out = subprocess.run(["nm", "-D", "--defined-only", G.lib.PROBE_LIB_PATH], capture_output=True, text=True).stdout
    assert "ltp_probe_random_access" in out
