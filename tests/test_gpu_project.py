"""Direction sets, tile projection (sh.comp) and reconstruction (sh_sum.comp) vs the oracle."""
import numpy as np
import pytest

import oracle as O
import vlb

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n", [64, 256, 1024, 1000])
def test_fibonacci_directions_bit_exact(ctx, n):
    ds = ctx.fibonacci(n)
    d, b = ds.export()
    od, ow = O.dirs_fibonacci(n)
    assert np.array_equal(d, od)
    ref = O.basis_matrix(od.astype(np.float64), ow, 3)
    assert np.max(np.abs(b - ref)) <= 1e-7 * np.max(np.abs(ref))


def test_equirect_directions_bit_exact(ctx):
    ds = ctx.equirect(64, 32)
    d, b = ds.export()
    t, bd, w = O.dirs_equirect(64, 32)
    assert np.array_equal(d, t)
    ref = O.basis_matrix(bd, w, 3)
    assert np.max(np.abs(b - ref)) <= 1e-7 * np.max(np.abs(ref))


def test_xzy_frame(ctx):
    d, b = ctx.fibonacci(128, vlb.FRAME_XZY).export()
    od, ow = O.dirs_fibonacci(128)
    ref = O.basis_matrix(od.astype(np.float64)[:, [0, 2, 1]], ow, 3)
    assert np.max(np.abs(b - ref)) <= 1e-7 * np.max(np.abs(ref))


@pytest.mark.parametrize("lmax", [2, 3])
@pytest.mark.parametrize("nprobes,S", [(1, 64), (37, 256), (700, 1024), (5, 100), (5, 65536), (343, 20000)])
def test_project_f32_matches_oracle(ctx, lmax, nprobes, S):
    """Includes tiles of few rows and many samples, projected in sample splits
    (ragged last split) whose partials are added in FP64."""
    ds = ctx.fibonacci(S)
    d, w = O.dirs_fibonacci(S)
    B = O.basis_matrix(d.astype(np.float64), w, lmax)
    rng = np.random.default_rng(nprobes * 31 + S)
    rad = rng.random((nprobes, 3, S)).astype(np.float32) * 5
    got = ctx.project(rad, nprobes, ds, lmax)
    ref = O.project(rad, nprobes, S, B)
    assert rel(got, ref) < 1e-5


def test_project_bf16_matches_oracle_on_rounded_input(ctx):
    torch = pytest.importorskip("torch")
    S, n = 1024, 300
    ds = ctx.fibonacci(S)
    d, w = O.dirs_fibonacci(S)
    B = O.basis_matrix(d.astype(np.float64), w, 2)
    rng = np.random.default_rng(4)
    rad = torch.from_numpy(rng.random((n, 3, S)).astype(np.float32) * 5).to(torch.bfloat16)
    bits = rad.view(torch.int16).numpy().copy()
    got = ctx.project(bits, n, ds, 2, dtype=vlb.DTYPE_BF16)
    ref = O.project(rad.float().numpy(), n, S, B)
    assert rel(got, ref) < 1e-5


def test_project_bf16_split_simt_matches_oracle(ctx):
    """BF16 tile whose sample count rules out the tensor-core kernel (not a
    multiple of 8), few rows: the CUDA-core kernel in sample splits."""
    torch = pytest.importorskip("torch")
    S, n = 30001, 7
    ds = ctx.fibonacci(S)
    d, w = O.dirs_fibonacci(S)
    B = O.basis_matrix(d.astype(np.float64), w, 3)
    rng = np.random.default_rng(5)
    rad = torch.from_numpy(rng.random((n, 3, S)).astype(np.float32) * 5).to(torch.bfloat16)
    bits = rad.view(torch.int16).numpy().copy()
    got = ctx.project(bits, n, ds, 3, dtype=vlb.DTYPE_BF16)
    ref = O.project(rad.float().numpy(), n, S, B)
    assert rel(got, ref) < 1e-5


@pytest.mark.parametrize("lmax", [2, 3])
@pytest.mark.parametrize("nprobes,S", [(1, 64), (43, 1000), (300, 1024), (5, 104), (7, 100), (100_000, 1024)])
def test_project_bf16_tensor_core_matches_oracle(ctx, lmax, nprobes, S):
    """BF16 tiles go through the tcgen05 kernel (S % 8 == 0) or the CUDA-core
    kernel (S = 100); hi/lo BF16 basis, FP32 accumulation."""
    torch = pytest.importorskip("torch")
    ds = ctx.fibonacci(S)
    d, w = O.dirs_fibonacci(S)
    B = O.basis_matrix(d.astype(np.float64), w, lmax)
    g = torch.Generator().manual_seed(nprobes + S + lmax)
    rad = (torch.rand((nprobes, 3, S), generator=g) * 5).to(torch.bfloat16)
    dev = rad.cuda().view(torch.int16)
    out = torch.empty((nprobes, vlb.k_of(lmax), 3), dtype=torch.float32, device="cuda")
    ctx.project(dev, nprobes, ds, lmax, dtype=vlb.DTYPE_BF16, out=out)
    ctx.synchronize()
    got = out.cpu().numpy()
    m = min(nprobes, 2000)  # the oracle checks a prefix of the large tile
    ref = O.project(rad[:m].float().numpy(), m, S, B)
    assert rel(got[:m], ref) < 1e-5
    assert np.isfinite(got).all()


def _split_bf16(torch, rad):
    """FP32 samples [n, 3, S] -> hi/lo BF16 pairs [n, 3, 2S] (hi, then the rounding of the remainder)."""
    hi = rad.to(torch.bfloat16)
    lo = (rad - hi.float()).to(torch.bfloat16)
    return torch.cat([hi, lo], dim=2).contiguous()


@pytest.mark.parametrize("lmax", [2, 3])
@pytest.mark.parametrize("nprobes,S", [(1, 64), (300, 1024), (5, 100), (7, 30001), (50_000, 256)])
def test_project_bf16_split_matches_fp32_oracle(ctx, lmax, nprobes, S):
    """Hi/lo BF16 pairs (the mixed-precision tile): tensor cores for S % 4 == 0
    (K = 2S against the split basis), CUDA cores otherwise.  The pair keeps
    ~16 mantissa bits of each FP32 sample, so the result is within 2e-5 of the
    FP64 projection of the FP32 samples themselves."""
    torch = pytest.importorskip("torch")
    ds = ctx.fibonacci(S)
    d, w = O.dirs_fibonacci(S)
    B = O.basis_matrix(d.astype(np.float64), w, lmax)
    g = torch.Generator().manual_seed(3 * nprobes + S + lmax)
    rad = torch.rand((nprobes, 3, S), generator=g) * 5
    dev = _split_bf16(torch, rad).cuda().view(torch.int16)
    out = torch.empty((nprobes, vlb.k_of(lmax), 3), dtype=torch.float32, device="cuda")
    ctx.project(dev, nprobes, ds, lmax, dtype=vlb.DTYPE_BF16_SPLIT, out=out)
    ctx.synchronize()
    got = out.cpu().numpy()
    m = min(nprobes, 2000)
    ref = O.project(rad[:m].numpy(), m, S, B)
    assert rel(got[:m], ref) < 2e-5
    assert np.isfinite(got).all()


def test_sh_eval_matches_reference_golden(ctx, golden):
    w, h = (int(v) for v in golden["recon_wh"])
    got = ctx.sh_eval_envmap(golden["coeffs"], 3, w, h, 1250.0)
    assert rel(got, golden["recon"]) < 1e-5


def test_project_then_eval_round_trip(ctx):
    rng = np.random.default_rng(8)
    coeffs = rng.normal(size=(16, 3)).astype(np.float32)
    img = ctx.sh_eval_envmap(coeffs, 3, 512, 256, 1.0)
    back = ctx.skybox_sh(img, vlb.SKY_ENVMAP, 512, 256, 3)
    assert rel(back, coeffs.astype(np.float64)) < 1e-4
