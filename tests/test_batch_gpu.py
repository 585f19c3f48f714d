"""Many robust meshes in one persistent launch: results equal the one-mesh evaluator's bit for bit.

The batched workload mirrors the uneven multi-mesh configuration at a small scale: noisy icospheres and tori with
random holes, one uniform query grid per mesh of a different size, plus degenerate members (a closed mesh with no
boundary, a single triangle, an empty query set).  Every tuner configuration, the captured CUDA graph and the
direct launch must produce the same bits as agwn_robust_eval on each mesh alone.
"""

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu


def build_meshes(dt, seed=0):
    rng = np.random.default_rng(seed)
    meshes = []
    for j, (kind, ntri, holes, side) in enumerate([("icosphere", 1300, 3, 24), ("torus", 3000, 7, 9),
                                                    ("icosphere", 500, 1, 17), ("torus", 800, 12, 30),
                                                    ("icosphere", 320, 0, 12), ("torus", 6000, 2, 0)]):
        v, i = synth.noisy_mesh(kind, ntri, holes, rng)
        b = synth.boundary_segments(v, i)
        q = synth.grid_queries(v.min(0), v.max(0), side) if side else np.zeros((0, 3))
        meshes.append((v.astype(dt), i, b.astype(dt), q.astype(dt)))
    # a single triangle (its boundary is its three edges)
    v1 = np.array([[0.1, -0.3, 0.2], [0.8, 0.4, -0.1], [-0.5, 0.6, 0.3]])
    i1 = np.array([0, 1, 2], np.int32)
    q1 = synth.grid_queries(v1.min(0), v1.max(0), 11)
    meshes.append((v1.astype(dt), i1, synth.boundary_segments(v1, i1).astype(dt), q1.astype(dt)))
    return meshes


@pytest.mark.parametrize("dt,policy", [(np.float32, "int64_grid"), (np.float64, "int128_grid"),
                                       (np.float64, "exact_float")])
def test_batch_equals_per_mesh(gwn, disp, dt, policy):
    torch = pytest.importorskip("torch")
    tdt = torch.float32 if dt == np.float32 else torch.float64
    meshes = build_meshes(dt)
    robust = [gwn.CudaRobustMeshGwn(disp, v, i, b, precision=policy) for v, i, b, _ in meshes]
    ref_out, ref_cnt = [], []
    for r, (_, _, _, q) in zip(robust, meshes):
        o = np.empty(len(q), dt)
        c = np.empty(len(q), np.int32)
        r.evaluate(q, o, c)
        ref_out.append(o)
        ref_cnt.append(c)
    pos = [torch.from_numpy(q).cuda() for *_, q in meshes]
    outs = [torch.full((len(q),), float("nan"), dtype=tdt, device="cuda") for *_, q in meshes]
    cnts = [torch.full((len(q),), -7, dtype=torch.int32, device="cuda") for *_, q in meshes]
    batch = gwn.CudaRobustBatch(disp, robust, pos, outs, cnts)
    info = batch.info()
    assert info["queries"] == sum(len(q) for *_, q in meshes)
    configs = [(128, 1, 256, 64), (256, 2, 1024, 64), (128, 2, 512, 64), (256, 1, 32, 64)]
    if all(r.info()["depth"] < 32 for r in robust):
        configs.append((256, 2, 256, 32))
    for cfg in configs:
        for o in outs:
            o.fill_(float("nan"))
        batch.set_config(*cfg)
        batch.run(graph=False)
        torch.cuda.synchronize()
        for k in range(len(meshes)):
            assert np.array_equal(outs[k].cpu().numpy(), ref_out[k]), (cfg, k)
            assert np.array_equal(cnts[k].cpu().numpy(), ref_cnt[k]), (cfg, k)
    # the tuner picks one of its candidates; the graph replays give the same bits
    tuned = batch.tune(repeats=1)
    assert tuned["candidates"] >= 12 and max(tuned["tune_ms"][:tuned["candidates"]]) > 0
    c = tuned["config"]
    assert (c["block"], c["k"]) in [(128, 1), (128, 2), (256, 1), (256, 2)]
    for rep in range(3):
        for o in outs:
            o.fill_(float("nan"))
        batch.run(graph=True)
        torch.cuda.synchronize()
        for k in range(len(meshes)):
            assert np.array_equal(outs[k].cpu().numpy(), ref_out[k]), (rep, k)
    batch.close()
    for r in robust:
        r.close()


def test_batch_errors(gwn, disp):
    torch = pytest.importorskip("torch")
    m32 = build_meshes(np.float32)[:2]
    m64 = build_meshes(np.float64)[:1]
    r32 = [gwn.CudaRobustMeshGwn(disp, v, i, b) for v, i, b, _ in m32]
    r64 = gwn.CudaRobustMeshGwn(disp, *m64[0][:3])
    q = torch.zeros((5, 3), dtype=torch.float32, device="cuda")
    o = torch.zeros(5, dtype=torch.float32, device="cuda")
    with pytest.raises(TypeError):
        gwn.CudaRobustBatch(disp, r32, [q.cpu(), q], [o, o])
    with pytest.raises(gwn.GwnError):  # mixed policies / scalar types
        gwn.CudaRobustBatch(disp, [r32[0], r64], [q, q.double()], [o, o.double()])
    with pytest.raises(ValueError):
        gwn.CudaRobustBatch(disp, r32, [q], [o])
    b = gwn.CudaRobustBatch(disp, r32, [q, q], [o, o])
    with pytest.raises(gwn.GwnError):
        b.set_config(512, 1, 256, 64)
    b.close()


@pytest.mark.parametrize("dt,policy,mode", [(np.float32, "int64_grid", "exact"), (np.float32, "int64_grid", "mixed"),
                                            (np.float64, "int64_grid", "mixed"), (np.float64, "int128_grid", "exact"),
                                            (np.float64, "exact_float", "exact")])
def test_batch_matches_oracle(gwn, disp, oracle, dt, policy, mode):
    """The batch against the CPU oracle (the reference's RobustMeshGwn rule) on a seeded sample of every mesh's
    queries: counts bit for bit; values within the exact tolerance (1e-12 double, 1e-6 float, as the golden tests),
    or in mixed mode within 1e-7 of FP64 (float outputs: plus two ulps of the value's rounding)."""
    torch = pytest.importorskip("torch")
    tdt = torch.float32 if dt == np.float32 else torch.float64
    meshes = build_meshes(dt, seed=3)
    robust = [gwn.CudaRobustMeshGwn(disp, v, i, b, precision=policy) for v, i, b, _ in meshes]
    pos = [torch.from_numpy(q).cuda() for *_, q in meshes]
    outs = [torch.full((len(q),), float("nan"), dtype=tdt, device="cuda") for *_, q in meshes]
    cnts = [torch.full((len(q),), -7, dtype=torch.int32, device="cuda") for *_, q in meshes]
    disp.set_robust_precision(mode)
    try:
        batch = gwn.CudaRobustBatch(disp, robust, pos, outs, cnts)
        batch.tune(repeats=1)
        batch.run(graph=True)
        torch.cuda.synchronize()
    finally:
        disp.set_robust_precision("exact")
    rng = np.random.default_rng(41)
    ulps = 0.0 if dt == np.float64 or mode == "exact" else 2 * 2.0 ** -23
    tol = (1e-12 if dt == np.float64 else 1e-6) if mode == "exact" else 1e-7
    checked = 0
    for k, (v, i, b, q) in enumerate(meshes):
        if len(q) == 0:
            continue
        pick = np.sort(rng.choice(len(q), size=min(len(q), 400), replace=False))
        gw, rc, rf = oracle.robust_eval(policy, v, i, b, q[pick])
        got_c = cnts[k].cpu().numpy()[pick]
        got = outs[k].cpu().numpy()[pick].astype(np.float64)
        assert np.array_equal(got_c, rc), (k, int(np.sum(got_c != rc)))
        ref = gw.astype(np.float64)
        err = np.abs(got - ref) - ulps * np.maximum(1, np.abs(ref))
        assert float(err.max()) <= tol, (k, float(err.max()))
        checked += len(pick)
    assert checked > 2000
    batch.close()
    for r in robust:
        r.close()
