"""The serving loops' latency histogram (ltpmg_gb300/csrc/ltp_histo.h): the
request-log server adds a run of requests with sorted arrivals in one call;
that must equal adding each request's latency alone (CPU, compiled here)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def test_sorted_run_histogram_equals_per_request_adds(tmp_path):
    exe = str(tmp_path / "histo_check")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(HERE, "histo", "histo_check.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
