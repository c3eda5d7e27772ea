"""nerfgb_render_rays_noalloc: the fused render for callers that cannot
allocate device memory (code inside a framework whose allocator has reserved
the GPU, as TensorFlow does at start-up). It must give the same maps as
nerfgb_render_rays with a caller-allocated workspace, call after call, even
though every call reuses one library-owned scratch array.

This file is named to be collected last."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return None if t is None else t.data_ptr()


def _render(ng, noalloc, nerf, rays, uc, uf, seed):
    lib = ng._lib.lib()
    R = rays[0].shape[0]
    Sc, Sf = nerf.params.sampling.N_coarse, nerf.params.sampling.N_fine
    out = [torch.full((R, 3), -1.0, device="cuda"), torch.full((R,), -1.0, device="cuda"),
           torch.full((R,), -1.0, device="cuda"), torch.full((R, 3), -1.0, device="cuda"),
           torch.full((R,), -1.0, device="cuda"), torch.full((R,), -1.0, device="cuda")]
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    pc, pf = nerf.coarse_model.packed(), nerf.fine_model.packed()
    args = [_ptr(pc), _ptr(pf), ng._lib.PREC_BF16, *map(_ptr, rays), _ptr(uc), _ptr(uf),
            ctypes.c_ulonglong(seed), R, Sc, Sf, 1, 1, 0, ng._lib.TRANS_LOGSUM, *map(_ptr, out)]
    if noalloc:
        rc = lib.nerfgb_render_rays_noalloc(*args, _ptr(err), stream)
    else:
        ws = torch.empty(lib.nerfgb_render_workspace_bytes(R, Sc, Sf), dtype=torch.uint8, device="cuda")
        rc = lib.nerfgb_render_rays(*args, _ptr(ws), _ptr(err), stream)
    torch.cuda.synchronize()
    assert rc == ng._lib.OK, ng._lib.status_name(rc)
    assert int(err.item()) == 0
    return out


def test_noalloc_matches_workspace_render_twice(ng):
    nerf = ng.NeRF(ng.make_params(), precision="bf16", seed=5)
    # Two calls in a row: a large one, then a smaller one with Philox uniforms,
    # so a stale intermediate from the first call would show in the second.
    for R, seed, explicit in ((1500, 11, True), (333, 12, False)):
        o, d, n, f = ng.synthetic.sphere_rays(R, seed)
        rays = [torch.from_numpy(x).cuda() for x in (o, d, n, f)]
        if explicit:
            rng = np.random.default_rng(seed)
            uc = torch.from_numpy(rng.random((R, 64), dtype=np.float32)).cuda()
            uf = torch.from_numpy(rng.random((R, 128), dtype=np.float32)).cuda()
        else:
            uc = uf = None
        got = _render(ng, True, nerf, rays, uc, uf, seed)
        want = _render(ng, False, nerf, rays, uc, uf, seed)
        for g, w in zip(got, want):
            # same kernels on the same inputs: identical bits (tolerance 0)
            assert torch.equal(g, w)
        assert float(got[3].min()) >= 0.0


def test_noalloc_rejects_requests_beyond_scratch(ng):
    """A request whose intermediates exceed the 16 MiB array is refused with
    NERFGB_E_SCRATCH_LIMIT, and its outputs are left untouched."""
    lib = ng._lib.lib()
    R = 4096
    need = lib.nerfgb_render_workspace_bytes(R, 64, 128)
    assert need > (16 << 20)
    nerf = ng.NeRF(ng.make_params(), precision="bf16", seed=5)
    o, d, n, f = ng.synthetic.sphere_rays(R, 3)
    rays = [torch.from_numpy(x).cuda() for x in (o, d, n, f)]
    outs = [torch.full((R, 3), -1.0, device="cuda"), torch.full((R,), -1.0, device="cuda"),
            torch.full((R,), -1.0, device="cuda")]
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    pc, pf = nerf.coarse_model.packed(), nerf.fine_model.packed()
    rc = lib.nerfgb_render_rays_noalloc(_ptr(pc), _ptr(pf), ng._lib.PREC_BF16, *map(_ptr, rays), None, None,
                                        ctypes.c_ulonglong(0), R, 64, 128, 1, 1, 0, ng._lib.TRANS_LOGSUM,
                                        None, None, None, *map(_ptr, outs), _ptr(err),
                                        torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == ng._lib.E_SCRATCH_LIMIT
    assert ng._lib.status_name(rc) == "NERFGB_E_SCRATCH_LIMIT"
    assert all(bool((t == -1.0).all()) for t in outs) and int(err.item()) == 0
