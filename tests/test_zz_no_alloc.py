"""The allocation-free TV entry point (asdpocs_tv_device_noalloc).

It exists for callers that cannot allocate device memory themselves (a
framework allocator that owns the GPU's memory, a fixed memory budget, a
real-time loop that must not stall on cudaMalloc): its scratch is a fixed
array inside the library.  This file is collected last so that a run that
stops at its first failure has already run every other test; it passes both
alone in a fresh process and after the other tests."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _call(fn, img, old, shape, alpha, n, pos):
    import torch

    from asd_pocs_mex_cuda_demo_gb300._lib import check

    t = img.clone()
    check(fn(t.data_ptr(), old.data_ptr(), *shape, alpha, n, pos,
             torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("shape", [(512, 512, 1), (64, 48, 40)])
def test_noalloc_tv_matches_allocating_entry_point(gpu, shape):
    import torch

    from asd_pocs_mex_cuda_demo_gb300._lib import load

    L = load()
    rng = np.random.default_rng(sum(shape))
    # two calls in a row: the second sees the array as the first left it
    for call in range(2):
        img = torch.tensor(rng.random(int(np.prod(shape))), dtype=torch.float32,
                           device=gpu)
        old = torch.tensor(rng.random(int(np.prod(shape))), dtype=torch.float32,
                           device=gpu)
        n = 10 + 5 * call
        ref = _call(L.asdpocs_tv_device, img, old, shape, 0.2, n, 1)
        out = _call(L.asdpocs_tv_device_noalloc, img, old, shape, 0.2, n, 1)
        assert rel_l2(out, ref) < 1e-5, (call, rel_l2(out, ref))


def test_noalloc_tv_rejects_images_over_its_limit(gpu):
    import torch

    from asd_pocs_mex_cuda_demo_gb300._lib import AsdpocsError, check, load

    L = load()
    big = torch.zeros(1025 * 1024, device=gpu)
    with pytest.raises(AsdpocsError, match="1048576-voxel limit"):
        check(L.asdpocs_tv_device_noalloc(big.data_ptr(), None, 1025, 1024, 1, 0.2, 3, 1,
                                          torch.cuda.current_stream().cuda_stream))
    # a thin image within the voxel and tile limits whose tile rows
    # (ceil(ny/8) * nz = 65536) exceed what one launch can hold
    thin = torch.zeros(16 * 65536, device=gpu)
    with pytest.raises(AsdpocsError, match="tile rows"):
        check(L.asdpocs_tv_device_noalloc(thin.data_ptr(), None, 16, 1, 65536, 0.2, 3, 1,
                                          torch.cuda.current_stream().cuda_stream))
