"""The serving loop (GB300Server*) through the C ABI.

Each request's result must be the same when it is served alone on an idle server and when it
is served in a mix: many requests in flight at once, batched into shared rounds on several
streams, with a table budget small enough that topologies are evicted and re-uploaded between
uses.  Results are also checked against the oracle: refine requests against the restated
EvalStencils, limit requests against the restated patch-point stencils + PatchMap +
EvalPatches (P, dPdu, dPdv), within 1e-6 x sum_j |w_j x_j| + 1e-6 per element for stencils and
1e-5 x max(sum |w x|, 1) for patch outputs (float rounding of the GPU patch points carries
into them).
"""
import numpy as np
import pytest

import oracle
from gpu_util import serving_bases, torch_cuda

N_POINTS = 4000


def _pool():
    from opensubdiv_gb300 import workloads
    return workloads.serving_pool(serving_bases(), n_topologies=8, cv_min=400, cv_max=4000, seed=99)


def _work(pool):
    """Two requests per topology (refine + limit) with host inputs; returns a list of dicts."""
    from opensubdiv_gb300 import workloads
    reqs = []
    for t in pool:
        cv = workloads.serving_control_values(t, seed=t["id"])
        n_out = len(t["refine"]["sizes"]) * t["length"]
        reqs.append(dict(topo=t, kind=0, cv=cv, n_out=n_out))
        f, u, v = workloads.serving_queries(t, N_POINTS, seed=100 + t["id"])
        reqs.append(dict(topo=t, kind=1, cv=cv, n_out=9 * N_POINTS, faces=f, u=u, v=v))
    return reqs


def _server(pool, budget, streams=3, plain=False):
    from opensubdiv_gb300.server import GB300Server
    s = GB300Server(budget, 1 << 30, streams=streams, max_requests_per_round=16, plain=plain)
    for t in pool:
        s.add_topology(t["id"], t["num_control"], t["length"], t["refine"], t["limit"])
    return s


def _table_bytes(t):
    r, lm = t["refine"], t["limit"]
    return (8 * len(r["sizes"]) + 8 * len(r["indices"]) + 8 * len(lm["pp_sizes"])
            + 8 * len(lm["pp_indices"]) + 4 * len(lm["patch_indices"]) + 12 * len(lm["params"])
            + 24 * len(lm["arrays"]) + 64 * len(lm["params"]) + 4096 * 16)


def _run_alone(server, reqs, torch):
    from opensubdiv_gb300.server import GB300Server, LIMIT
    outs = []
    for q in reqs:
        out = np.zeros(q["n_out"], np.float32)
        r = GB300Server.request(q["topo"]["id"], q["kind"], q["cv"], out,
                                *((q["faces"], q["u"], q["v"]) if q["kind"] == LIMIT else ()))
        server.wait(server.submit(r))
        outs.append(out)
    return outs


def _oracle(q):
    t = q["topo"]
    L = t["length"]
    if q["kind"] == 0:
        r = t["refine"]
        n = len(r["sizes"])
        out = np.zeros(n * L, np.float32)
        oracle.eval_stencils(q["cv"], (0, L, L), [out], [(0, L, L)], r["sizes"], r["offsets"],
                             r["indices"], [r["weights"]], threads=8)
        bound = 1e-6 * oracle.stencil_abs_scale(q["cv"], (0, L, L), r["sizes"], r["offsets"],
                                                r["indices"], r["weights"]) + 1e-6
        return out, bound
    lm = t["limit"]
    npp = len(lm["pp_sizes"])
    ps = np.zeros(npp * 3, np.float32)
    oracle.eval_stencils(q["cv"], (0, 3, L), [ps], [(0, 3, 3)], lm["pp_sizes"], lm["pp_offsets"],
                         lm["pp_indices"], [lm["pp_weights"]], threads=8)
    pm = oracle.PatchMap(lm["arrays"], lm["params"], lm["triangular"])
    handles = pm.find(q["faces"], q["u"], q["v"])
    hit = handles[:, 0] >= 0
    coords = oracle.make_coords(handles[hit], q["u"][hit], q["v"][hit])
    m = int(hit.sum())
    refs = [np.zeros(m * 3, np.float32) for _ in range(3)]
    oracle.eval_patches(ps, (0, 3, 3), refs, [(0, 3, 3)] * 3, coords, lm["arrays"],
                        lm["patch_indices"], lm["params"], threads=8)
    A = oracle.abs_scale(ps, (0, 3, 3), 3, coords, lm["arrays"], lm["patch_indices"],
                         lm["params"])
    n = len(q["faces"])
    out = np.zeros((3, n, 3), np.float32)
    bound = np.full((3, n, 3), 1e-6)
    for k in range(3):
        out[k][hit] = refs[k].reshape(m, 3)
        bound[k][hit] = 1e-5 * np.maximum(A[k].reshape(m, 3), 1.0)
    return out.ravel(), bound.ravel()


@pytest.mark.gpu
def test_server_requests_alone_match_the_oracle():
    torch = torch_cuda()
    pool = _pool()
    reqs = _work(pool)
    s = _server(pool, budget=sum(_table_bytes(t) for t in pool) * 2)
    outs = _run_alone(s, reqs, torch)
    st = s.stats()
    s.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["evictions"] == 0
    for q, out in zip(reqs, outs):
        ref, bound = _oracle(q)
        assert np.all(np.abs(out - ref) <= bound), (q["topo"]["id"], q["kind"])


@pytest.mark.gpu
def test_server_results_same_alone_and_in_the_mix():
    """Alone on an idle server vs all at once (three times over, shuffled) on a server whose
    table budget holds only a few topologies: same results within the tolerance."""
    torch = torch_cuda()
    from opensubdiv_gb300.server import GB300Server, LIMIT
    pool = _pool()
    reqs = _work(pool)
    alone_srv = _server(pool, budget=sum(_table_bytes(t) for t in pool) * 2)
    alone = _run_alone(alone_srv, reqs, torch)
    alone_srv.close()
    budget = max(_table_bytes(t) for t in pool) * 3
    mix_srv = _server(pool, budget=budget, streams=3)
    order = np.random.default_rng(1).permutation(np.tile(np.arange(len(reqs)), 3))
    outs, cvs, pins = [], [], []
    for i in order:
        q = reqs[i]
        cv = torch.from_numpy(q["cv"]).pin_memory()
        out = torch.zeros(q["n_out"], pin_memory=True)
        extra = ()
        if q["kind"] == LIMIT:
            extra = tuple(torch.from_numpy(a).pin_memory() for a in (q["faces"], q["u"], q["v"]))
        pins.append((cv, out, extra))
        outs.append(GB300Server.request(q["topo"]["id"], q["kind"], cv, out, *extra))
    # arrivals 20 us apart: requests join rounds while earlier rounds are in flight
    lat = mix_srv.replay(outs, np.arange(len(outs)) * 20e-6)
    st = mix_srv.stats()
    mix_srv.close()
    assert st["completed"] == len(order) and st["failed"] == 0
    assert st["evictions"] > 0 and st["uploads"] > len(pool)  # re-admissions happened
    assert st["rounds"] < len(order)  # requests shared rounds
    assert np.all(lat > 0)
    exact = 0
    for i, (cv, out, _) in zip(order, pins):
        ref, bound = _oracle(reqs[i]) if i == order[0] else (None, None)
        a = alone[i]
        b = out.numpy()
        exact += int(np.array_equal(a, b))
        # same result alone and in the mix, within the tolerance stated for each request kind
        tol = (1e-6 * np.maximum(np.abs(a), 1.0)) if reqs[i]["kind"] == 0 else \
            (1e-5 * np.maximum(np.abs(a), 1.0))
        assert np.all(np.abs(a - b) <= tol), (int(i), reqs[i]["kind"])
        if ref is not None:
            assert np.all(np.abs(b - ref) <= bound)
    print(f"{exact}/{len(order)} results bit-identical alone vs in the mix; stats {st}")


@pytest.mark.gpu
def test_plain_server_matches_batched():
    torch = torch_cuda()
    pool = _pool()[:4]
    reqs = _work(pool)
    budget = sum(_table_bytes(t) for t in pool) * 2
    a = _run_alone(_server(pool, budget), reqs, torch)
    b = _run_alone(_server(pool, budget, plain=True), reqs, torch)
    for q, x, y in zip(reqs, a, b):
        assert np.all(np.abs(x - y) <= 1e-5 * np.maximum(np.abs(x), 1.0)), q["kind"]


@pytest.mark.gpu
def test_server_rejects_bad_requests():
    torch_cuda()
    from opensubdiv_gb300.evaluator import GB300Error
    from opensubdiv_gb300.server import GB300Server
    pool = _pool()[:1]
    s = _server(pool, budget=_table_bytes(pool[0]) * 2)
    cv = np.zeros(pool[0]["num_control"] * pool[0]["length"], np.float32)
    out = np.zeros(10, np.float32)
    with pytest.raises(GB300Error):
        s.submit(GB300Server.request(12345, 0, cv, out))  # unknown topology
    with pytest.raises(GB300Error):
        s.submit(GB300Server.request(pool[0]["id"], 7, cv, out))  # unknown kind
    big = np.zeros(300_000_000, np.int32)  # query arrays larger than the 1 GiB arena
    with pytest.raises(GB300Error):
        s.submit(GB300Server.request(pool[0]["id"], 1, cv, out, big, big.view(np.float32),
                                     big.view(np.float32)))
    with pytest.raises(GB300Error):  # a topology larger than the budget
        small = GB300Server(1 << 20, 1 << 24)
        t = pool[0]
        small.add_topology(t["id"], t["num_control"], t["length"], t["refine"], t["limit"])
    s.close()


@pytest.mark.gpu
def test_server_topologies_from_table_cache_files(tmp_path):
    """Topologies registered from table-cache files (mapped, re-read on re-admission) give the
    results of topologies registered from host arrays, under a budget that forces evictions."""
    torch = torch_cuda()
    from opensubdiv_gb300.server import GB300Server, write_table_cache
    pool = _pool()[:5]
    reqs = _work(pool)
    ref_srv = _server(pool, budget=sum(_table_bytes(t) for t in pool) * 2)
    expect = _run_alone(ref_srv, reqs, torch)
    ref_srv.close()
    srv = GB300Server(max(_table_bytes(t) for t in pool) * 2, 1 << 30, streams=3,
                      max_requests_per_round=16, pin_host_tables=True)
    for t in pool:
        path = tmp_path / f"topo{t['id']}.gbtc"
        write_table_cache(path, t["num_control"], t["length"], t["refine"], t["limit"])
        srv.add_topology_from_cache(t["id"], path)
    for _ in range(2):  # twice round: the second pass re-admits evicted topologies
        got = _run_alone(srv, reqs, torch)
        for q, a, b in zip(reqs, expect, got):
            assert np.array_equal(a, b), (q["topo"]["id"], q["kind"])
    st = srv.stats()
    srv.close()
    assert st["evictions"] > 0 and st["failed"] == 0
