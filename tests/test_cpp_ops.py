"""The C++ operator surface (include/trax_ops.hpp): it compiles against the
C-ABI, and the chain program fails loudly without a GPU."""
import pytest

from cpp_chain import compile_chain, run_chain
from golden_util import fixtures, load


@pytest.fixture(scope="module")
def chain(tmp_path_factory):
    from trax_gb300 import build
    build.build()
    return compile_chain(str(tmp_path_factory.mktemp("cpp")))


def test_chain_without_gpu_fails_loudly(chain, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    b, cfg, grid, _ = load(fixtures()[0])
    p, out = run_chain(chain, b, cfg, grid, str(tmp_path))
    assert p.returncode == 1 and out is None
    assert "trax_ctx_create" in p.stderr
