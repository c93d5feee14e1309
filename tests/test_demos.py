"""The scenario command line (particlesimulation_gb300/demos/pmgb_demos.cpp) builds against the
facade and, like the reference's main (source/main.cpp:23-81), rejects an unknown option with
exit code 1 (no GPU involved)."""
import subprocess


def test_demos_build_and_unknown_option():
    from particlesimulation_gb300 import build
    exe = build.build_demos()
    r = subprocess.run([exe, "no-such-demo"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Unknown option: no-such-demo" in r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
