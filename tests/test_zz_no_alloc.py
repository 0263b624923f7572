"""gb_recip_energy_noalloc against gb_box_reciprocal on the same structure
factors, called through the C ABI on caller-owned device arrays.

The entry point keeps its scratch in a fixed device array of the library and
allocates nothing; its sum runs in the order of the box path, so the two
agree to the last bit on every call.  This file is
collected last so that it also runs after the rest of the suite in one
process; it passes alone as well.
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    from gomc_gb300 import engine
    from gomc_gb300.config import SimConfig
    from gomc_gb300.systems import spce_water_box
    lib = engine.lib(build_if_missing=True)
    box = engine.Box(spce_water_box(2000, 39.1, seed=3),
                     SimConfig(temperature=298.0, rcut=10.0, tolerance=1e-5))
    kv = box.kvectors()
    ref = box.box_reciprocal(is_new_volume=False)
    dev = torch.device("cuda:0")
    arrs = [torch.tensor(kv[k], dtype=torch.float64, device=dev)
            for k in ("sumRref", "sumIref", "prefact")]
    yield torch, lib, arrs, ref, dev
    box.close()


def test_noalloc_matches_box_reciprocal_twice(setup):
    torch, lib, (sR, sI, pf), ref, dev = setup
    K = sR.numel()
    out = torch.empty(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        out.fill_(float("nan"))
        rc = lib.gb_recip_energy_noalloc(sR.data_ptr(), sI.data_ptr(),
                                         pf.data_ptr(), K, out.data_ptr(),
                                         stream)
        assert rc == 0, lib.gb_last_error(None)
        torch.cuda.synchronize(dev)
        e = out.item()
        # the same sum in the same order as gb_box_reciprocal: equal to the
        # last bit (the relative error is reported if it is not)
        assert e == ref, (e, ref, abs(e - ref) / abs(ref))


def test_noalloc_rejects_k_beyond_scratch(setup):
    torch, lib, (sR, sI, pf), ref, dev = setup
    from gomc_gb300._lib import RECIP_NOALLOC_MAX_K
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    # rejected before anything is launched, so the short arrays are never read
    rc = lib.gb_recip_energy_noalloc(sR.data_ptr(), sI.data_ptr(),
                                     pf.data_ptr(), RECIP_NOALLOC_MAX_K + 1,
                                     out.data_ptr(), None)
    assert rc == 4  # GB_ERR_CAPACITY
    assert b"GB_RECIP_NOALLOC_MAX_K" in lib.gb_last_error(None)
    torch.cuda.synchronize(dev)
    assert out.item() == 0.0
