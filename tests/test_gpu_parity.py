"""GPU parity: the engine through its C ABI against the exact oracle, the
reference's golden vectors and the rknn-inf restatement.  Results are
integer id sets: equality is bit-exact."""
import json
import os

import numpy as np
import pytest

import datagen
import oracle as O

pytestmark = pytest.mark.gpu

MODES = ("fp64", "fp32")


@pytest.fixture(scope="module")
def c1(engine):
    ds = datagen.uniform(1000, 10000, seed=1, nq=10, k=5)
    return ds, engine.Index.of(ds), O.Oracle.of(ds)


def test_handmade_cases(engine, golden_dir):
    for c in json.load(open(os.path.join(golden_dir, "handmade.json"))):
        idx = engine.Index(np.array(c["fxy"], np.float32), np.array(c["uxy"], np.float32),
                           c["fid"], c["uid"])
        keys = list(c["expect"])
        for mode in MODES:
            for key in keys:
                q, k = map(int, key.split(","))
                assert idx.query(q, k, mode).tolist() == c["expect"][key], (c["name"], key, mode)
            qs = [int(kk.split(",")[0]) for kk in keys]
            ks = [int(kk.split(",")[1]) for kk in keys]
            got = idx.query_batch(qs, ks, mode)
            assert [g.tolist() for g in got] == [c["expect"][kk] for kk in keys], (c["name"], mode)
        idx.close()


def test_config1_single_and_batch(c1):
    ds, idx, o = c1
    want = [o.query(int(q), 5) for q in ds.queries]
    for mode in MODES:
        for q, w in zip(ds.queries, want):
            assert np.array_equal(idx.query(int(q), 5, mode), w), (q, mode)
        got = idx.query_batch(ds.queries, 5, mode)
        assert all(np.array_equal(g, w) for g, w in zip(got, want)), mode


def test_integer_twin_against_naive_golden(engine, golden_dir):
    g = json.load(open(os.path.join(golden_dir, "naive_int_1k10k.json")))
    z = np.load(os.path.join(golden_dir, "uniform_int_1k10k.npz"))
    idx = engine.Index(z["fxy"], z["uxy"], z["fid"], z["uid"])
    o = O.Oracle(z["fxy"], z["uxy"], z["fid"], z["uid"])
    qs = [int(q) for q in g["ids"]]
    for mode in MODES:
        got = idx.query_batch(qs, g["k"], mode)
        for q, res in zip(qs, got):
            assert np.array_equal(res, o.query(q, g["k"])), (q, mode)
            # strict-< only adds users that rknn-naive drops on an exact tie
            assert set(g["ids"][str(q)]) <= set(res.tolist())


def test_inf_golden_superset(engine, golden_dir):
    g = json.load(open(os.path.join(golden_dir, "inf_float_1k10k.json")))
    z = np.load(os.path.join(golden_dir, "uniform_1k10k.npz"))
    idx = engine.Index(z["fxy"], z["uxy"], z["fid"], z["uid"])
    for q, ids in g["ids"].items():
        res = idx.query(int(q), g["k"], "fp32")
        assert set(res.tolist()) <= set(ids)


def test_mixed_k_batch(engine):
    ds = datagen.uniform(5000, 50000, seed=12, nq=300, k=1)
    rng = np.random.default_rng(3)
    ks = rng.integers(1, 41, size=ds.queries.shape[0]).astype(np.int32)
    idx = engine.Index.of(ds)
    o = O.Oracle.of(ds)
    got32 = idx.query_batch(ds.queries, ks, "fp32")
    got64 = idx.query_batch(ds.queries[:60], ks[:60], "fp64")
    for i, q in enumerate(ds.queries):
        w = o.query(int(q), int(ks[i]))
        assert np.array_equal(got32[i], w), (q, ks[i])
        if i < 60:
            assert np.array_equal(got64[i], w), (q, ks[i])


def test_gaussmix_ties_and_duplicates(engine):
    ds = datagen.gaussmix(20_000, 400_000, seed=3, nq=200, k=10)
    idx = engine.Index.of(ds)
    o = O.Oracle.of(ds)
    got, st = idx.query_batch(ds.queries, 10, "fp32", stats=True)
    for q, res in zip(ds.queries, got):
        assert np.array_equal(res, o.query(int(q), 10)), q
    assert st["rechecks"] > 0          # exact ties reached the exact predicate
    got64 = idx.query_batch(ds.queries[:50], 10, "fp64")
    for q, res in zip(ds.queries[:50], got64):
        assert np.array_equal(res, o.query(int(q), 10)), q


def test_street_large_k(engine):
    ds = datagen.street(nu=200_000, nf=2000, seed=4, nq=80)
    idx = engine.Index.of(ds)
    o = O.Oracle.of(ds)
    got = idx.query_batch(ds.queries, ds.ks, "fp32")
    for q, k, res in zip(ds.queries, ds.ks, got):
        assert np.array_equal(res, o.query(int(q), int(k))), (q, k)


def test_result_set_sizes(engine):
    """Few facilities, many users: result sets of tens to tens of thousands of
    ids, sorted by a warp in registers (<= 32), by a warp in shared memory
    (<= 512), by the block in shared memory (<= 4096) and by radix passes
    through the result pool above that."""
    ds = datagen.uniform(200, 100_000, seed=21, nq=60, k=1)
    o = O.Oracle.of(ds)
    ks = np.array([1, 8, 20, 2] * 15, np.int32)
    idx = engine.Index.of(ds)
    got = idx.query_batch(ds.queries, ks, "fp32")
    sizes = [r.size for r in got]
    assert min(sizes) <= 512 < max(sizes) and max(sizes) > 4096
    for q, k, res in zip(ds.queries, ks, got):
        assert np.array_equal(res, o.query(int(q), int(k))), (int(q), int(k))
    mid = datagen.uniform(2000, 100_000, seed=23, nq=60, k=1)
    om = O.Oracle.of(mid)
    idx3 = engine.Index.of(mid)
    km = np.array([1, 2, 3, 5] * 15, np.int32)
    got = idx3.query_batch(mid.queries, km, "fp32")
    sizes = [r.size for r in got]
    for lo, hi in ((32, 64), (64, 128), (128, 256), (256, 512)):
        assert any(lo < n <= hi for n in sizes), (lo, hi, sorted(sizes))
    for q, k, res in zip(mid.queries, km, got):
        assert np.array_equal(res, om.query(int(q), int(k))), (int(q), int(k))
    idx3.close()
    small = datagen.uniform(20_000, 100_000, seed=22, nq=40, k=1)
    os_ = O.Oracle.of(small)
    idx2 = engine.Index.of(small)
    got = idx2.query_batch(small.queries, 3, "fp32")
    assert max(r.size for r in got) <= 32
    for q, res in zip(small.queries, got):
        assert np.array_equal(res, os_.query(int(q), 3)), int(q)
    idx.close()
    idx2.close()


def _device_results(idx, nq):
    """The last device batch's (ids, offsets) copied to the host."""
    import torch

    class _Dev:
        def __init__(self, ptr, n, typestr):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                             "version": 3, "strides": None}

    idx.sync()
    ids_p, off_p = idx.device_results()
    off = torch.as_tensor(_Dev(off_p, nq + 1, "<i4"), device="cuda").cpu().numpy().astype(np.int64)
    n = int(off[-1])
    ids = torch.as_tensor(_Dev(ids_p, max(n, 1), "<i4"), device="cuda").cpu().numpy()[:n] if n else np.zeros(0, np.int32)
    return [ids[off[i]:off[i + 1]] for i in range(nq)]


@pytest.mark.parametrize("filt", ["slice", "inf"])
def test_device_batch_with_understated_kmax(engine, filt):
    """rknn_query_batch_device: q and k already on the device; a k above the
    stated kmax is still answered exactly."""
    import torch
    ds = datagen.uniform(3000, 40000, seed=31, nq=120, k=1)
    o = O.Oracle.of(ds)
    rng = np.random.default_rng(5)
    ks = rng.integers(1, 41, ds.queries.shape[0]).astype(np.int32)
    idx = engine.Index.of(ds, filter=filt)
    d_q = torch.from_numpy(ds.queries.astype(np.int32)).cuda()
    d_k = torch.from_numpy(ks).cuda()
    for kmax in (40, 8):
        idx.query_batch_device(d_q.data_ptr(), d_k.data_ptr(), len(ks), kmax, "fp32")
        got = _device_results(idx, len(ks))
        for q, k, res in zip(ds.queries, ks, got):
            assert np.array_equal(res, o.query(int(q), int(k))), (int(q), int(k), kmax)
    idx.close()


def test_fused_and_separate_verification_agree(engine, monkeypatch):
    """Batches that fit two warps a query are verified inside the slice
    filter (fused); RKNN_FUSE=0 at index creation keeps the separate
    verification kernel.  Both give the oracle's ids, including queries with
    more than 4096 candidates (left over to the verification kernel in the
    fused batch), mixed k (several filter launches counted by one last-block
    counter) and a device batch whose kmax understates some k."""
    import torch
    ds = datagen.uniform(300, 60_000, seed=51, nq=80, k=1)
    o = O.Oracle.of(ds)
    rng = np.random.default_rng(8)
    ks = rng.integers(1, 30, ds.queries.shape[0]).astype(np.int32)
    want = [o.query(int(q), int(k)) for q, k in zip(ds.queries, ks)]
    got = {}
    for fuse in ("1", "0"):
        monkeypatch.setenv("RKNN_FUSE", fuse)
        idx = engine.Index.of(ds)
        res, st = idx.query_batch(ds.queries, ks, "fp32", stats=True)
        assert (st["fused_slots"] > 0) == (fuse == "1"), st["fused_slots"]
        if fuse == "1":
            assert st["fused_slots"] < len(ks)        # some queries were left over
            assert st["candidates"] > 4096
        got[fuse] = res
        for q, k, r, w in zip(ds.queries, ks, res, want):
            assert np.array_equal(r, w), (int(q), int(k), fuse)
        d_q = torch.from_numpy(ds.queries.astype(np.int32)).cuda()
        d_k = torch.from_numpy(ks).cuda()
        idx.query_batch_device(d_q.data_ptr(), d_k.data_ptr(), len(ks), 4, "fp32")
        for q, k, r, w in zip(ds.queries, ks, _device_results(idx, len(ks)), want):
            assert np.array_equal(r, w), (int(q), int(k), fuse, "device")
        idx.close()
    assert all(np.array_equal(a, b) for a, b in zip(got["1"], got["0"]))


def test_snapshot_index_gives_the_same_ids(engine, tmp_path):
    """An index saved as a snapshot and reopened (rknn_index_save /
    rknn_index_open, through the command line as well) answers as the
    original."""
    import subprocess
    ds = datagen.uniform(2000, 30_000, seed=61, nq=12, k=4)
    o = O.Oracle.of(ds)
    idx = engine.Index.of(ds)
    p = str(tmp_path / "idx.rkx")
    idx.save(p)
    fxy, fid, uxy, uid = engine.snapshot_read(p)
    assert np.array_equal(fxy, ds.fxy) and np.array_equal(fid, ds.fid)
    assert np.array_equal(uxy, ds.uxy) and np.array_equal(uid, ds.uid)
    idx2 = engine.Index.open(p)
    a = idx.query_batch(ds.queries, 4, "fp32")
    b = idx2.query_batch(ds.queries, 4, "fp32")
    for q, x, y in zip(ds.queries, a, b):
        assert np.array_equal(x, y) and np.array_equal(x, o.query(int(q), 4)), int(q)
    cli = os.path.join(os.path.dirname(engine.__file__), "rknn-gb300")
    q = int(ds.queries[0])
    r = subprocess.run([cli, "-if", p, "-k", "4", "-q", str(q), "--log", str(tmp_path / "log")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.loadtxt(tmp_path / "log" / f"fp64_k4_q{q}.txt", dtype=np.int64, ndmin=1)
    assert np.array_equal(got, o.query(q, 4))
    idx.close()
    idx2.close()


def test_flat_batches_into_page_locked_ids(engine):
    """query_batch_flat keeps one page-locked id buffer: from its second call
    the finalize kernel writes the ids into it directly.  Batches that fit,
    one that outgrows it (capacity error, larger buffer, retry) and smaller
    ones after give the same ids as the per-query form and the oracle."""
    ds = datagen.uniform(2000, 100_000, seed=41, nq=50, k=1)
    o = O.Oracle.of(ds)
    idx = engine.Index.of(ds)
    for k in (1, 1, 2, 30, 30, 3, 3):
        ids, off = idx.query_batch_flat(ds.queries, k, "fp32")
        ref = idx.query_batch(ds.queries, k, "fp32")
        assert off[-1] == sum(r.size for r in ref)
        for i, r in enumerate(ref):
            assert np.array_equal(ids[off[i]:off[i + 1]], r), (i, k)
        for i in range(0, len(ds.queries), 10):
            assert np.array_equal(ref[i], o.query(int(ds.queries[i]), k)), (i, k)
    idx.close()


@pytest.mark.parametrize("cta", ["256", "128", "0"])
def test_zone_bisectors_match_port(engine, monkeypatch, cta):
    """Same grid, same rules: the zone kernel builds rknn-inf's bisector set
    in the same order as the CPU restatement does -- the one-block kernel
    (small batches and single queries) at 256 and at 128 threads, and the
    one-warp kernel (cta=0) alike."""
    monkeypatch.setenv("RKNN_ZONE_CTA", cta)
    for nf, nu, k in ((1000, 10000, 5), (20000, 200000, 10), (20000, 200000, 3), (20000, 200000, 25)):
        ds = datagen.uniform(nf, nu, seed=31 + k, nq=40, k=k)
        idx = engine.Index.of(ds, filter="inf")
        info = idx.info()
        port = O.InfPort(ds.fxy, ds.uxy, grid=(info["fgrid_x0"], info["fgrid_y0"], info["fgrid_inv"],
                                               info["fgrid_gx"], info["fgrid_gy"]))
        idx.query_batch(ds.queries, k, "fp32")
        same = 0
        ports = []
        for slot, q in enumerate(ds.queries):
            gb, flags = idx.last_zone(slot)
            pb, _, _ = port.query(int(q), k, verify=False)
            ports.append(pb)
            same += np.array_equal(gb, pb)
            assert flags & 7 == 0
        assert same == len(ds.queries), (nf, k, same, cta)
        # one query per launch (the plain form)
        for q, pb in list(zip(ds.queries, ports))[:8]:
            idx.query(int(q), k, "fp64")
            gb, flags = idx.last_zone(0)
            assert np.array_equal(gb, pb) and flags & 7 == 0, (int(q), k, cta)
        idx.close()


def test_full_scale_checksum(engine):
    """Config 2 sizes (100k facilities, 1M users): every facility as a query;
    without distance ties each user lies in exactly k result sets, so the
    result sizes sum to k * |U|."""
    ds = datagen.uniform(100_000, 1_000_000, seed=2, nq=1000, k=10)
    idx = engine.Index.of(ds)
    allq = np.arange(ds.nf, dtype=np.int32)
    for k in (1, 10):
        got = idx.query_batch(allq, k, "fp32")
        assert sum(len(g) for g in got) == k * ds.nu, k
    sub = ds.queries[:200]
    a = idx.query_batch(sub, 10, "fp32")
    b = idx.query_batch(sub, 10, "fp64")
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    o = O.Oracle.of(ds)
    for q, res in zip(sub[:20], a[:20]):
        assert np.array_equal(res, o.query(int(q), 10)), q


def test_argument_errors(engine, c1):
    ds, idx, _ = c1
    with pytest.raises(engine.RkNNError) as e:
        idx.query(ds.nf, 3)
    assert e.value.status == 1
    with pytest.raises(engine.RkNNError) as e:
        idx.query(0, 0)
    assert e.value.status == 1
    with pytest.raises(engine.RkNNError) as e:
        idx.query_batch([0, -1], 3)
    assert e.value.status == 1


def test_edge_cases(engine):
    rng = np.random.default_rng(8)
    f = rng.uniform(0, 100, (30, 2)).astype(np.float32)
    u = rng.uniform(0, 100, (500, 2)).astype(np.float32)
    # no users
    idx = engine.Index(f, np.zeros((0, 2), np.float32))
    assert idx.query(3, 2).size == 0
    # one facility: every user
    idx = engine.Index(f[:1], u)
    assert idx.query(0, 1).size == 500
    # k >= |F|: every user
    idx = engine.Index(f, u)
    assert idx.query(5, 30).size == 500 and idx.query(5, 31, "fp32").size == 500
    # all users on one point, duplicated facilities
    f2 = np.concatenate([f, f[:5]])
    u2 = np.repeat(u[:1], 300, 0)
    idx = engine.Index(f2, u2)
    o = O.Oracle(f2, u2)
    for q in (0, 2, 31, 33):
        for k in (1, 2, 6):
            assert np.array_equal(idx.query(q, k), o.query(q, k)), (q, k)


def test_command_line_drop_in(engine, golden_dir, tmp_path):
    """`rknn-gb300 -if <file> -k <k> -q <index>` as the reference's binaries are
    called: the reference's text format in, its summary lines out, and the
    result set in log/<mode>_k<k>_q<q>.txt (sorted user ids, one per line)."""
    import subprocess
    z = np.load(os.path.join(golden_dir, "uniform_int_1k10k.npz"))
    g = json.load(open(os.path.join(golden_dir, "naive_int_1k10k.json")))
    ds = datagen.Dataset(z["fxy"], z["uxy"], z["fid"], z["uid"], z["queries"], z["ks"], "golden_int")
    path = tmp_path / "points.txt"
    datagen.write_text(str(path), ds)
    o = O.Oracle(z["fxy"], z["uxy"], z["fid"], z["uid"])
    cli = os.path.join(os.path.dirname(engine.__file__), "rknn-gb300")
    k = g["k"]
    qs = [int(q) for q in g["ids"]][:4]
    for mode in MODES:
        for q in qs:
            r = subprocess.run([cli, "-if", str(path), "-k", str(k), "-q", str(q), "-al", "inf",
                                "--mode", mode, "--log", str(tmp_path / "log")],
                               capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
            assert f"Loaded {ds.nf} facilities and {ds.nu} users." in r.stdout
            want = o.query(q, k)
            assert f"Found {want.size} RkNN results." in r.stdout
            got = np.loadtxt(tmp_path / "log" / f"{mode}_k{k}_q{q}.txt", dtype=np.int64, ndmin=1)
            assert np.array_equal(got, want), (q, mode)
            assert set(g["ids"][str(q)]) <= set(got.tolist())
    # several queries in one batch, slice filter
    r = subprocess.run([cli, "-if", str(path), "-k", str(k), "--queries", ",".join(map(str, qs)),
                        "--filter", "slice", "--mode", "fp32", "--log", str(tmp_path / "log2")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for q in qs:
        got = np.loadtxt(tmp_path / "log2" / f"fp32_k{k}_q{q}.txt", dtype=np.int64, ndmin=1)
        assert np.array_equal(got, o.query(q, k)), q


def test_zone_boundary_vertex_test(engine):
    """The zone-boundary vertex test (rknn_index_opts.zone_vertex_test = 1:
    every zone-boundary vertex considered, instead of rknn-inf's count-(k-1)
    and extreme boundary vertices) gives the oracle's results in both modes,
    batched and one query per launch, both zone kernels."""
    ds = datagen.uniform(20000, 200000, seed=51, nq=40, k=10)
    o = O.Oracle.of(ds)
    for k in (1, 5, 10, 25):
        want = [o.query(int(q), k) for q in ds.queries]
        with engine.Index.of(ds, filter="inf", zone_vertex_test="boundary") as idx:
            for mode in MODES:
                got = idx.query_batch(ds.queries, k, mode)
                assert all(np.array_equal(g, w) for g, w in zip(got, want)), (k, mode)
            for q, w in list(zip(ds.queries, want))[:5]:
                assert np.array_equal(idx.query(int(q), k, "fp64"), w), (int(q), k)
