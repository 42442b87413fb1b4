"""Bake service (vlb_service_*): continuous batching on a worker thread.

Every result must equal vlb_bake of the same request bit for bit, whatever
the batch it landed in; a relight must equal vlb_bake of the original probes
with the relight's sun and sky, whether its kept hits were still resident or
had been evicted (then it bakes in full).
"""
import threading

import numpy as np
import pytest

import vlb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(ctx):
    rng = np.random.default_rng(21)
    scenes = []
    for i, nb in enumerate((8, 64, 700)):
        pos, idx, alb = vlb.synth_box_scene(300 + i, nb)
        sc = ctx.scene(pos, idx, alb)
        b = sc.bounds()
        scenes.append((sc, b))
    dsets = {64: ctx.fibonacci(64), 256: ctx.fibonacci(256)}
    sky = ctx.sky(vlb.synth_cubemap(9, 32), 32)

    def probes(b, n):
        return (b[:3] + rng.random((n, 3)) * (b[3:] - b[:3])).astype(np.float32)

    return dict(scenes=scenes, dsets=dsets, sky=sky, probes=probes, rng=rng)


def _params(w, S, sun, prec=vlb.PREC_MIXED, lmax=2, intensity=5.0):
    return vlb.bake_params(w["dsets"][S], lmax, prec, sun, sun_intensity=intensity, sky=w["sky"])


@pytest.mark.parametrize("prec", [vlb.PREC_MIXED, vlb.PREC_FP32, vlb.PREC_FUSED, vlb.PREC_BF16])
def test_service_matches_bake(ctx, world, prec):
    w = world
    svc = vlb.Service(ctx, lmax=2, precision=prec, max_batch_probes=3000)
    reqs = []
    for i in range(24):
        sc, b = w["scenes"][i % 3]
        n = int(w["rng"].integers(1, 1200))
        S = 64 if i % 2 else 256
        p = _params(w, S, vlb.synth_sun(i), prec)
        pr = w["probes"](b, n)
        reqs.append((svc.submit(sc, pr, p), sc, pr, p))
    for t, sc, pr, p in reqs:
        got, lat = svc.wait(t)
        assert lat > 0
        assert np.array_equal(got, ctx.bake(sc, pr, p))
    st = svc.stats()
    assert st["completed"] == 24 and st["failed"] == 0 and 1 <= st["batches"] <= 24
    svc.close()


@pytest.mark.parametrize("prec", [vlb.PREC_FUSED, vlb.PREC_MIXED])
def test_service_slices_large_requests(ctx, world, prec):
    """slice_probes = 97: requests of up to 1500 probes bake in slices that
    share batches with the requests behind them; every result, and every
    relight of a sliced kept bake, equals vlb_bake bit for bit."""
    w = world
    svc = vlb.Service(ctx, lmax=2, precision=prec, max_batch_probes=400, slice_probes=97)
    reqs = []
    for i in range(12):
        sc, b = w["scenes"][i % 3]
        n = int(w["rng"].integers(1, 1500))
        S = 64 if i % 2 else 256
        p = _params(w, S, vlb.synth_sun(200 + i), prec)
        pr = w["probes"](b, n)
        t = svc.submit(sc, pr, p, keep_hits=i % 3 == 0)
        reqs.append((t, sc, pr, p))
        if i % 3 == 0:  # queued right behind its (sliced) bake
            q = _params(w, S, vlb.synth_sun(300 + i), prec, intensity=2.5)
            reqs.append((svc.submit(None, None, q, relight_of=t), sc, pr, q))
    for t, sc, pr, p in reqs:
        got, lat = svc.wait(t)
        assert lat > 0
        assert np.array_equal(got, ctx.bake(sc, pr, p))
    st = svc.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["relights"] == 4 and st["relights_rebaked"] == 0
    total = sum(len(pr) for _, _, pr, _ in reqs)
    assert st["batches"] >= -(-total // 400) and st["probes"] == total
    svc.close()


def test_service_threads_and_relights(ctx, world):
    w = world
    svc = vlb.Service(ctx, lmax=2, precision=vlb.PREC_MIXED, max_batch_probes=4000)
    out, errs = [], []

    def client(k):
        try:
            rng = np.random.default_rng(100 + k)
            sc, b = w["scenes"][k % 3]
            for j in range(4):
                n = int(rng.integers(16, 800))
                pr = (b[:3] + rng.random((n, 3)) * (b[3:] - b[:3])).astype(np.float32)
                p = _params(w, 256, vlb.synth_sun(10 * k + j))
                t = svc.submit(sc, pr, p, keep_hits=True)
                p2 = _params(w, 256, vlb.synth_sun(1000 + 10 * k + j), intensity=3.0)
                t2 = svc.submit(None, None, p2, relight_of=t)
                out.append((svc.wait(t)[0], ctx_lock_bake(sc, pr, p)))
                out.append((svc.wait(t2)[0], ctx_lock_bake(sc, pr, p2)))
        except Exception as e:  # pragma: no cover - reported below
            errs.append(e)

    lock = threading.Lock()

    def ctx_lock_bake(sc, pr, p):  # the user context is externally synchronised
        with lock:
            return ctx.bake(sc, pr, p)

    th = [threading.Thread(target=client, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    assert len(out) == 32
    for a, b in out:
        assert np.array_equal(a, b)
    st = svc.stats()
    assert st["relights"] == 16 and st["completed"] == 32
    svc.close()


def test_service_eviction_and_release(ctx, world):
    w = world
    sc, b = w["scenes"][2]
    pr = [w["probes"](b, 300) for _ in range(3)]
    one = 300 * 256 * 8 + 300 * 12  # one kept-hit set
    tile = 300 * 256 * 3 * 2 + 300 * (12 + 4 + 16 + 9 * 12)
    svc = vlb.Service(ctx, budget_bytes=one + 2 * tile + one // 2, lmax=2, precision=vlb.PREC_MIXED,
                      max_batch_probes=300, max_inflight=1)
    p = [_params(w, 256, vlb.synth_sun(50 + i)) for i in range(3)]
    t = [svc.submit(sc, pr[i], p[i], keep_hits=True) for i in range(3)]
    for i in range(3):
        svc.wait(t[i])
    st = svc.stats()
    assert st["evictions"] >= 1
    # relight every set: the evicted ones bake in full, same bits
    q = _params(w, 256, vlb.synth_sun(77), intensity=2.0)
    r = [svc.submit(None, None, q, relight_of=t[i]) for i in range(3)]
    for i in range(3):
        assert np.array_equal(svc.wait(r[i])[0], ctx.bake(sc, pr[i], q))
    st = svc.stats()
    assert st["relights_rebaked"] >= 1 and st["bytes_peak"] <= one + 2 * tile + one // 2
    # release: a later relight bakes in full
    svc.release(t[2])
    r2 = svc.submit(None, None, p[0], relight_of=t[2])
    assert np.array_equal(svc.wait(r2)[0], ctx.bake(sc, pr[2], p[0]))
    svc.close()


def test_service_refusals(ctx, world):
    w = world
    sc, b = w["scenes"][0]
    svc = vlb.Service(ctx, budget_bytes=1 << 20, lmax=2, precision=vlb.PREC_MIXED)
    p = _params(w, 256, vlb.synth_sun(3))
    with pytest.raises(vlb.VlbError) as e:
        svc.submit(sc, w["probes"](b, 4096), p)  # 4096 x 256 x 6 B > 1 MiB
    assert e.value.status == vlb.ERR_OOM
    with pytest.raises(vlb.VlbError) as e:
        svc.submit(None, None, p, relight_of=12345)
    assert e.value.status == vlb.ERR_INVALID
    assert vlb.lib.vlb_service_wait(svc.h, 999, 0, None, None) == vlb.ERR_INVALID
    pr = w["probes"](b, 10)
    t = svc.submit(sc, pr, p)
    got, _ = svc.wait(t)
    assert np.array_equal(got, ctx.bake(sc, pr, p))
    with pytest.raises(vlb.VlbError):  # collected once
        svc.wait(t)
    svc.close()


def test_service_destroy_finishes_pending(ctx, world):
    w = world
    sc, b = w["scenes"][1]
    svc = vlb.Service(ctx, lmax=2, precision=vlb.PREC_MIXED)
    for i in range(6):
        svc.submit(sc, w["probes"](b, 500), _params(w, 64, vlb.synth_sun(i)))
    svc.close()  # must return after the six bakes, without error


def test_context_close_with_requests_in_flight():
    """Closing a context while its service still has submitted requests: the
    service finishes them and stops before the scenes, direction sets and
    skies those requests name are destroyed (no use after free)."""
    c = vlb.Context(0)
    pos, idx, alb = vlb.synth_box_scene(77, 300)
    sc = c.scene(pos, idx, alb)
    ds = c.fibonacci(256)
    sky = c.sky(vlb.synth_cubemap(3, 32), 32)
    svc = vlb.Service(c, lmax=2, precision=vlb.PREC_FP32, max_batch_probes=2000)
    rng = np.random.default_rng(5)
    b = sc.bounds()
    for i in range(12):
        p = vlb.bake_params(ds, 2, vlb.PREC_FP32, vlb.synth_sun(i), sky=sky)
        svc.submit(sc, (b[:3] + rng.random((1500, 3)) * (b[3:] - b[:3])).astype(np.float32), p)
    c.close()
    assert svc.h is None and sc.h is None and ds.h is None and c.h is None
    # the device is still usable afterwards
    c2 = vlb.Context(0)
    sc2 = c2.scene(pos, idx, alb)
    out = c2.bake(sc2, np.float32([[0.5, 0.5, 0.5]]), vlb.bake_params(c2.fibonacci(64), 2, vlb.PREC_FP32,
                                                                      vlb.synth_sun(1)))
    assert np.isfinite(out).all()
    c2.close()
