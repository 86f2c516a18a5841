"""The C-ABI from a plain C99 caller (tests/c/abi_probe.c): the header
compiles as strict C, the library links, the host-only calls answer without
a GPU, and context creation without a device returns a status and a message
instead of crashing."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "trax_gb300")


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    from trax_gb300 import build
    build.build()
    exe = os.path.join(str(tmp_path_factory.mktemp("c")), "abi_probe")
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror",
                    "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_probe.c"),
                    "-L" + LIBDIR, "-ltrax_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe],
                   check=True)
    return exe


def test_c_caller_host_calls_and_loud_context_failure(probe):
    import torch
    p = subprocess.run([probe], capture_output=True, text=True, timeout=120)
    assert "FAIL" not in p.stdout, p.stdout
    assert p.returncode == 0, p.stdout + p.stderr
    if not torch.cuda.is_available():
        assert "status 7:" in p.stdout  # TRAX_ERR_NO_DEVICE
