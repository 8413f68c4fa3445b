"""The public headers from C: a C99 program (tests/c/host_example.c) compiles
with -Wall -Wextra -Werror against include/, links against both libraries,
and runs its host-only calls (no GPU needed)."""
import os
import subprocess

from conftest import ROOT


def test_c99_program_compiles_links_and_runs(tmp_path):
    from nbots_gb300 import _lib as L
    L.lib()  # built
    pkg = os.path.dirname(L.GPU_SO)
    exe = tmp_path / "host_example"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "host_example.c"), "-o", str(exe),
           "-L" + pkg, "-lnbots_gpu", "-lnbots_host", "-Wl,-rpath," + pkg]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("ok "), (r.returncode, r.stdout, r.stderr)
