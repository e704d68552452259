"""The continuous-batching render server: every request served in a concurrent
mix of sizes, meshes and cameras renders exactly as it renders alone through
Scene::render (coverage and depth bit-exact, colour within COLOUR_TOL_LSB);
admission respects the device-memory budget."""
import math
import threading

import numpy as np
import pytest

from draw_gb300 import scenes as S
from helpers import COLOUR_TOL_LSB, compare, describe

pytestmark = pytest.mark.gpu


def _pool():
    """Three meshes, two textures, and a list of (object index, w, h, camera, light) requests."""
    meshes = [S.mesh_for_tris("torus", 3000), S.mesh_for_tris("sphere", 8000), S.mesh_for_tris("torus", 20000)]
    texs = [S.value_noise_checker(256, 256, 5), S.value_noise_checker(128, 128, 6, comps=3)]
    objs = []
    for i, (pos, nrm, uv, tri) in enumerate(meshes):
        mat = S.Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, i % 2, (i + 1) % 2)
        objs.append(S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(S._tris9(tri), 0)], [mat]))
    rng = np.random.Generator(np.random.PCG64(42))
    reqs = []
    for k in range(24):
        oi = int(rng.integers(0, 3))
        w, h = [(64, 64), (160, 90), (256, 256), (333, 200), (512, 300)][int(rng.integers(0, 5))]
        az, el, dist = rng.uniform(0, 2 * math.pi), rng.uniform(0.1, 1.0), rng.uniform(2.5, 4.0)
        cam = (dist * math.cos(el) * math.sin(az), dist * math.sin(el), dist * math.cos(el) * math.cos(az))
        light = [(3.0 * math.sin(az + 1), 4.0, 3.0 * math.cos(az + 1))]
        reqs.append((oi, w, h, cam, light, [2, 5, 32][k % 3], [float("inf"), 100000.0][k % 2]))
    return objs, texs, reqs


def _alone(objs, texs, reqs):
    """Reference frames: each request rendered alone through Scene/Canvas on its own context."""
    from draw_gb300 import renderer as R

    ctx = R.Context(0)
    tm = [R.TextureMap(t.img, t.width, t.height, t.comps, ctx) for t in texs]
    obs = [R.upload_object(o, tm, ctx) for o in objs]
    out = []
    for oi, w, h, cam, light, e, clear in reqs:
        sc = R.Scene(w, h, ctx)
        sc.camera.reset(cam, tuple(-c for c in cam), float(np.float32(w) / np.float32(h)), -0.5, -100.0, 60.0)
        sc.set_lights(light)
        sc.set_exponent(e)
        sc.add_obj(obs[oi])
        cv = R.Canvas(w, h, ctx)
        cv.init_depth(clear)
        sc.render(cv)
        out.append(cv.read())
    ctx.close()
    return out


def test_server_mix_equals_alone(gpu_ctx):
    from draw_gb300 import renderer as R

    objs, texs, reqs = _pool()
    ref = _alone(objs, texs, reqs)
    ctx = R.Context(0)
    tm = [R.TextureMap(t.img, t.width, t.height, t.comps, ctx) for t in texs]
    obs = [R.upload_object(o, tm, ctx) for o in objs]
    srv = R.Server(ctx, budget_bytes=1 << 30, max_batch=8, streams=3)
    tickets = [None] * len(reqs)

    def submit(part):
        for k in part:
            oi, w, h, cam, light, e, clear = reqs[k]
            tickets[k] = srv.submit(R.Server.request(obs[oi], w, h, cam, tuple(-c for c in cam), -0.5, -100.0, 60.0,
                                                     light, e, clear))

    th = [threading.Thread(target=submit, args=(range(i, len(reqs), 2),)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k, (oi, w, h, *_r) in enumerate(reqs):
        bgra, depth, lat = srv.wait(tickets[k], w, h, read=True)
        p = compare(ref[k], (bgra, depth), reqs[k][6])
        assert p.ok and p.colour_max_lsb <= COLOUR_TOL_LSB, f"request {k}: {describe(p)}"
        assert lat > 0
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["error"] == 0
    assert st["batches"] < len(reqs)  # requests were batched together
    srv.close()
    ctx.close()


def test_server_large_frames_in_the_mix(gpu_ctx, oracle_lib):
    """The serving configuration's large requests: 1920x1080 and 3840x2160 frames
    of a 1M-triangle sphere and a 2M-triangle torus, submitted together with
    256^2 and 512^2 frames of small meshes. Each result equals the same request
    rendered alone, and the large frames equal the oracle's render."""
    from draw_gb300 import renderer as R
    from helpers import oracle_render_many

    meshes = [S.mesh_for_tris("sphere", 1_000_000), S.mesh_for_tris("torus", 2_000_000),
              S.mesh_for_tris("torus", 5_000), S.mesh_for_tris("sphere", 20_000)]
    assert meshes[0][3].shape[0] >= 1_000_000 and meshes[1][3].shape[0] >= 1_900_000
    texs = [S.value_noise_checker(512, 512, 11), S.value_noise_checker(1024, 1024, 12)]
    objs = []
    for i, (pos, nrm, uv, tri) in enumerate(meshes):
        mat = S.Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, i % 2, i % 2)
        objs.append(S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(S._tris9(tri), 0)], [mat]))
    rng = np.random.Generator(np.random.PCG64(77))
    sizes = [(1920, 1080, 0), (3840, 2160, 0), (3840, 2160, 1), (1920, 1080, 1)]
    reqs = []
    for k in range(16):
        if k % 4 == 1:
            w, h, oi = sizes[k // 4]
        else:
            w, h = [(256, 256), (512, 512)][k % 2]
            oi = 2 + (k % 3 == 0)
        az, el, dist = rng.uniform(0, 2 * math.pi), rng.uniform(0.1, 1.0), rng.uniform(2.6, 4.0)
        cam = (dist * math.cos(el) * math.sin(az), dist * math.sin(el), dist * math.cos(el) * math.cos(az))
        light = [(3.0 * math.sin(az + 1), 4.0, 3.0 * math.cos(az + 1))]
        reqs.append((oi, w, h, cam, light, 2, float("inf")))
    ref = _alone(objs, texs, reqs)
    large = [k for k, r in enumerate(reqs) if r[1] >= 1920]
    descs = []
    for k in large:
        oi, w, h, cam, light, e, clear = reqs[k]
        descs.append(S.SceneDesc(w, h, cam_pos=cam, cam_dir=tuple(-c for c in cam), near=-0.5, far=-100.0,
                                 fov_x=60.0, lights=np.array(light, np.float32), exponent=e, clear_depth=clear,
                                 textures=texs, objects=[objs[oi]]))
    oref = dict(zip(large, oracle_render_many(descs)))
    ctx = R.Context(0)
    tm = [R.TextureMap(t.img, t.width, t.height, t.comps, ctx) for t in texs]
    obs = [R.upload_object(o, tm, ctx) for o in objs]
    srv = R.Server(ctx, budget_bytes=8 << 30, max_batch=16, streams=3)
    tickets = []
    for oi, w, h, cam, light, e, clear in reqs:
        tickets.append(srv.submit(R.Server.request(obs[oi], w, h, cam, tuple(-c for c in cam), -0.5, -100.0, 60.0,
                                                   light, e, clear)))
    for k, (oi, w, h, *_r) in enumerate(reqs):
        bgra, depth, _lat = srv.wait(tickets[k], w, h, read=True)
        p = compare(ref[k], (bgra, depth), reqs[k][6])
        assert p.ok, f"request {k} ({w}x{h}) vs alone: {describe(p)}"
        if k in oref:
            q = compare(oref[k], (bgra, depth), reqs[k][6])
            assert q.ok and q.n_covered > 0, f"request {k} ({w}x{h}) vs oracle: {describe(q)}"
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["error"] == 0
    srv.close()
    ctx.close()


def test_server_admission_respects_budget(gpu_ctx):
    from draw_gb300 import renderer as R

    objs, texs, _ = _pool()
    ctx = R.Context(0)
    tm = [R.TextureMap(t.img, t.width, t.height, t.comps, ctx) for t in texs]
    ob = R.upload_object(objs[1], tm, ctx)
    frame_bytes = 256 * 256 * 16
    budget = 24 << 20
    srv = R.Server(ctx, budget_bytes=budget, max_batch=16, streams=2)
    # a frame that can never fit is refused at submission
    with pytest.raises(R.DrawError) as e:
        srv.submit(R.Server.request(ob, 4096, 4096, (0, 1, 3), (0, -1, -3), -0.5, -100.0, 60.0, [(2, 4, 3)]))
    assert e.value.status == 7
    ts = [srv.submit(R.Server.request(ob, 256, 256, (0.2 * k, 1, 3), (-0.2 * k, -1, -3), -0.5, -100.0, 60.0,
                                      [(2, 4, 3)], discard=True)) for k in range(40)]
    for t in ts:
        srv.wait(t)
    st = srv.stats()
    assert st["completed"] == 40 and st["error"] == 0
    assert 0 < st["peak_bytes"] <= budget
    assert frame_bytes * 40 > budget  # the requests did not fit at once
    srv.close()
    ctx.close()


def test_server_failures_injected_on_the_host(gpu_ctx):
    """Host-side fault injection (no GPU fault): a request whose buffer
    allocation is made to fail completes with DG_E_OOM while the requests
    around it render; a pending request cancelled before admission completes
    with DG_E_CANCELLED; malformed requests are refused at submission; and
    buffers of finished requests are reused from the pool (fewer allocations
    than requests)."""
    from draw_gb300 import renderer as R

    objs, texs, reqs = _pool()
    ref = _alone(objs, texs, reqs[:8])
    ctx = R.Context(0)
    tm = [R.TextureMap(t.img, t.width, t.height, t.comps, ctx) for t in texs]
    obs = [R.upload_object(o, tm, ctx) for o in objs]
    srv = R.Server(ctx, budget_bytes=1 << 30, max_batch=4, streams=1)

    def request(k, **kw):
        oi, w, h, cam, light, e, clear = reqs[k]
        return R.Server.request(obs[oi], w, h, cam, tuple(-c for c in cam), -0.5, -100.0, 60.0, light, e, clear,
                                **kw)

    # malformed requests
    for bad in (dict(width=0), dict(height=70000), dict(nlights=0), dict(object=99)):
        q = request(0)
        for k, v in bad.items():
            setattr(q, k, v)
        with pytest.raises(R.DrawError) as e:
            srv.submit(q)
        assert e.value.status == 1, bad
    # a burst of requests: the scheduler admits them in batches of 4 on one stream, so
    # the later ones are still pending when the injections and the cancel arrive
    blocker = [srv.submit(request(k % 8, discard=True)) for k in range(64)]
    tickets = [srv.submit(request(k)) for k in range(8)]
    srv.inject_alloc_failure(tickets[3])
    srv.cancel(tickets[5])
    with pytest.raises(R.DrawError):
        srv.cancel(10 ** 9)  # unknown ticket
    for t in blocker:
        srv.wait(t)
    for k, t in enumerate(tickets):
        oi, w, h, *_r = reqs[k]
        if k in (3, 5):
            with pytest.raises(R.DrawError) as e:
                srv.wait(t, w, h, read=True)
            assert e.value.status == (7 if k == 3 else 10)
            continue
        bgra, depth, _lat = srv.wait(t, w, h, read=True)
        p = compare(ref[k], (bgra, depth), reqs[k][6])
        assert p.ok, f"request {k}: {describe(p)}"
    with pytest.raises(R.DrawError):
        srv.cancel(tickets[0])  # done already
    st = srv.stats()
    assert st["error"] == 0
    assert st["allocations"] < len(blocker) + len(tickets) - 2  # buffers came back from the pool
    srv.close()
    ctx.close()
