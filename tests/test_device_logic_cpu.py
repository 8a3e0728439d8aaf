"""Code of the library checked on the CPU with g++ (no GPU needed): pk_narrow.cuh (device code
compiled for the host) and pk_events.h (the host-side event dispatcher)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_heap_order_and_clustered_support(tmp_path):
    exe = tmp_path / "check_narrow"
    src = os.path.join(ROOT, "tests", "cpp", "check_narrow.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", src, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "heap_mismatch=0 support_mismatch_f64=0 support_mismatch_f32=0 uv_mismatch_f64=0 uv_mismatch_f32=0" in r.stdout
    assert "box_mismatch=0" in r.stdout


def test_event_dispatcher_rules(tmp_path):
    exe = tmp_path / "check_events"
    src = os.path.join(ROOT, "tests", "cpp", "check_events.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", src, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "event_check_failures=0" in r.stdout
