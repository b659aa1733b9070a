"""crt_sort_pairs_noalloc through the C ABI: the stable radix sort for callers
that cannot allocate device memory where they sort (cudaMalloc synchronises
the device; plugin hosts may forbid allocation; a hot path must not fail with
out-of-memory).  Its scratch is a fixed device array inside libcrt.so, so
results must equal crt_sort_pairs' exactly, call after call (the array keeps
the previous call's contents).  This file is collected last on purpose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(torch, rng, n, bits, with_vals):
    hi = 1 << bits
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 4] = keys[0]  # a long run of equal keys: stability matters
    rng.shuffle(keys)
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    vin = None
    if with_vals:
        vin = torch.from_numpy(rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.int32)).cuda()
    return kin, vin


def test_sort_pairs_noalloc_matches_sort_pairs(cuda):
    import crt
    torch = cuda
    rng = np.random.default_rng(2024)
    # two calls in a row on the shared scratch: a large one, then a smaller one
    # with explicit values and a different key width
    for n, bits, with_vals in ((crt.SORT_NOALLOC_MAX_PAIRS, 30, False), (70_001, 32, True)):
        kin, vin = _case(torch, rng, n, bits, with_vals)
        ka, va = torch.empty_like(kin), torch.empty_like(kin)
        kb, vb = torch.empty_like(kin), torch.empty_like(kin)
        crt.sort_pairs(kin, vin, ka, va, key_bits=bits)
        crt.sort_pairs_noalloc(kin, vin, kb, vb, key_bits=bits)
        torch.cuda.synchronize()
        assert torch.equal(ka, kb), f"keys differ (n={n})"
        assert torch.equal(va, vb), f"values differ (n={n})"
        order = np.argsort(kin.cpu().numpy().view(np.uint32), kind="stable")
        expect = order.astype(np.int32) if vin is None else vin.cpu().numpy()[order]
        assert np.array_equal(vb.cpu().numpy(), expect)


def test_sort_pairs_noalloc_rejects_oversize(cuda):
    import crt
    torch = cuda
    n = crt.SORT_NOALLOC_MAX_PAIRS + 1
    k = torch.zeros(n, dtype=torch.int32, device="cuda")
    with pytest.raises(crt.CrtError) as e:
        crt.sort_pairs_noalloc(k, None, torch.empty_like(k), torch.empty_like(k))
    assert e.value.status == 1 and "CRT_SORT_NOALLOC_MAX_PAIRS" in str(e.value)
