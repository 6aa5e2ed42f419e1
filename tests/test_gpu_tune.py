"""GPU test of the plan autotuner: it produces an entry, later handles use
it (and stay correct), and the text cache round-trips."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bss():
    import torch
    import blockstructuredsolvers_gb300 as bss
    assert torch.cuda.is_available()
    return bss


def test_autotune_entry_is_used_and_correct(bss, tmp_path):
    import torch
    bss.autotune_clear()
    assert bss.autotune_lookup(32, torch.float64, "mixed") is None
    e = bss.autotune(32, torch.float64, "mixed", N_probe=2048)
    assert e["wave_mult_x4"] in (2, 4, 8, 16) and e["seq_cutoff"] >= 2 and e["chain_blocks"] >= 16
    assert e["single_ms"] > 0 and e["batch_ms"] > 0
    assert bss.autotune_lookup(32, torch.float64, "mixed") == e
    rng = np.random.default_rng(1)
    A, B, d = O.gen_shifted_family(rng, 3000, 32, 1)
    data = bss.initialize_batched(3000, 32, torch.float64, precision="mixed")
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    info = bss.get_info(data)
    assert info["coarsest_blocks"] <= e["seq_cutoff"]
    x = download_x(data, 3000)
    assert O.rel_residual(A, B, x, d) <= 1e-12
    path = tmp_path / "tune.txt"
    bss.autotune_save(path)
    bss.autotune_clear()
    assert bss.autotune_lookup(32, torch.float64, "mixed") is None
    bss.autotune_load(path)
    assert bss.autotune_lookup(32, torch.float64, "mixed") == e
    bss.autotune_clear()
