"""Generate the golden vectors under tests/golden/ by running the reference's
own CPU binaries (built by `make -C oracle ref` from the reference sources).

Run in a container that has the reference sources; the GPU machine does not, and
the tests only read the committed fixtures.

    python tests/golden/make_golden.py

Fixtures:
  naive_int_1k10k.json   rknn-naive result ids (k=5, 10 queries) on the integer
                         twin of the 1k-facility / 10k-user uniform workload
  naive_int_10k100k.json rknn-naive result ids (k=10, 8 queries) on a 10k/100k
                         integer workload (inputs regenerated from the seed and
                         checked by checksum)
  inf_float_1k10k.json   rknn-inf result ids and bisector counts (k=5, 10
                         queries) on the float32 1k/10k workload; rknn-inf
                         over-reports, so these are supersets of the exact sets
  handmade.json          known-answer cases written out by hand, each with the
                         output of both reference binaries
  *.npz                  the small input sets themselves
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "rt-rknn_gb300"))
import datagen  # noqa: E402

REF = os.path.join(REPO, "oracle", "_ref")


def run_ref(binary: str, path: str, q: int, k: int):
    out = subprocess.run([os.path.join(REF, binary), "-if", path, "-k", str(k),
                          "-q", str(q)], capture_output=True, text=True, check=True).stdout
    ids = sorted(int(l.split()[1]) for l in out.splitlines() if l.startswith("ID "))
    found = [l for l in out.splitlines() if l.startswith("Found ")]
    nb = [int(l.split(":")[1]) for l in out.splitlines()
          if l.startswith("Total bisectors created")]
    count = int(found[0].split()[1]) if found else -1
    assert count == len(ids), (binary, count, len(ids))
    return ids, (nb[0] if nb else None)


def checksum(ds) -> str:
    h = hashlib.sha256()
    for a in (ds.fxy, ds.uxy, ds.fid, ds.uid):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def save_npz(name, ds):
    np.savez_compressed(os.path.join(HERE, name), fxy=ds.fxy, uxy=ds.uxy,
                        fid=ds.fid, uid=ds.uid, queries=ds.queries, ks=ds.ks)


def dataset(fxy, uxy, fid=None, uid=None):
    fxy = np.asarray(fxy, np.float32)
    uxy = np.asarray(uxy, np.float32)
    nf, nu = len(fxy), len(uxy)
    return datagen.Dataset(fxy, uxy,
                           np.asarray(fid if fid is not None else np.arange(nf), np.int32),
                           np.asarray(uid if uid is not None else np.arange(nf, nf + nu), np.int32))


def handmade():
    """Small known-answer cases.  Expected strict-< answers are written by
    hand from the geometry; the reference outputs are recorded beside them."""
    cases = []
    # 1. exact tie: user (20,10) is equidistant from facilities (10,10) and
    #    (30,10).  strict-<: nothing is strictly nearer for either query, so the
    #    user is a R1NN of both.  rknn-naive breaks the tie by (x,y,id).
    cases.append(dict(name="tie_pair", fxy=[[10, 10], [30, 10]], uxy=[[20, 10], [12, 10]],
                      fid=[0, 1], uid=[100, 101],
                      expect={"0,1": [100, 101], "1,1": [100]}))
    # 2. vertical and horizontal bisectors (rknn-inf/inf.h:158-168): facilities
    #    on the query's row and column.  User (60,65) is equidistant (d2=325)
    #    from the query and two other facilities: a strict-< R1NN.
    cases.append(dict(name="axis_bisectors",
                      fxy=[[50, 50], [70, 50], [50, 80], [30, 50], [50, 20]],
                      uxy=[[55, 55], [61, 50], [59, 50], [50, 66], [50, 64], [41, 50],
                           [39, 50], [50, 36], [50, 34], [60, 65]],
                      fid=list(range(5)), uid=list(range(10, 20)),
                      expect={"0,1": [10, 12, 14, 15, 17, 19], "0,2": [10, 11, 12, 13, 14, 15, 16, 17, 18, 19]}))
    # 3. one facility: no bisector at all, every user is a result (rknn-inf-gpu
    #    returns nothing here, rknn-inf-gpu/inf_kernel.cu:76-78).
    cases.append(dict(name="single_facility", fxy=[[5, 5]], uxy=[[1, 1], [9, 9], [5, 6]],
                      fid=[0], uid=[7, 8, 9], expect={"0,1": [7, 8, 9], "0,3": [7, 8, 9]}))
    # 4. k >= |F|: every user is a result for every query.
    cases.append(dict(name="k_ge_nf", fxy=[[0, 0], [10, 0], [0, 10]],
                      uxy=[[1, 1], [9, 1], [1, 9], [5, 5]], fid=[0, 1, 2], uid=[3, 4, 5, 6],
                      expect={"0,3": [3, 4, 5, 6], "1,5": [3, 4, 5, 6], "2,2": [3, 5, 6]}))
    # 5. a second facility at the query's own position is never strictly nearer.
    cases.append(dict(name="coincident_facility", fxy=[[10, 10], [10, 10], [40, 10]],
                      uxy=[[12, 10], [10, 4], [30, 10], [26, 10]], fid=[0, 1, 2],
                      uid=[5, 6, 7, 8], expect={"0,1": [5, 6], "1,1": [5, 6], "2,1": [7, 8]}))
    out = []
    with tempfile.TemporaryDirectory() as td:
        for c in cases:
            ds = dataset(c["fxy"], c["uxy"], c["fid"], c["uid"])
            p = os.path.join(td, c["name"] + ".txt")
            datagen.write_text(p, ds, integer=True)
            ref = {}
            for key in c["expect"]:
                q, k = map(int, key.split(","))
                ref[key] = {"naive": run_ref("rknn-naive-ids", p, q, k)[0],
                            "inf": run_ref("rknn-inf-ids", p, q, k)[0]}
            c["reference"] = ref
            out.append(c)
    return out


def main():
    if not os.path.exists(os.path.join(REF, "rknn-naive-ids")):
        subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle"), "ref"])
    with tempfile.TemporaryDirectory() as td:
        # integer twin, 1k/10k, k=5
        ds = datagen.uniform(1000, 10000, seed=1, nq=10, k=5, integer=True)
        p = os.path.join(td, "int.txt")
        datagen.write_text(p, ds, integer=True)
        res = {str(int(q)): run_ref("rknn-naive-ids", p, int(q), 5)[0] for q in ds.queries}
        save_npz("uniform_int_1k10k.npz", ds)
        json.dump({"k": 5, "binary": "rknn-naive", "ids": res,
                   "sha256": checksum(ds)}, open(os.path.join(HERE, "naive_int_1k10k.json"), "w"))

        # float32, 1k/10k, k=5: rknn-inf (superset of the exact answer)
        ds = datagen.uniform(1000, 10000, seed=1, nq=10, k=5)
        p = os.path.join(td, "float.txt")
        datagen.write_text(p, ds)
        res, nb = {}, {}
        for q in ds.queries:
            ids, b = run_ref("rknn-inf-ids", p, int(q), 5)
            res[str(int(q))] = ids
            nb[str(int(q))] = b
        save_npz("uniform_1k10k.npz", ds)
        json.dump({"k": 5, "binary": "rknn-inf", "ids": res, "bisectors": nb,
                   "sha256": checksum(ds)}, open(os.path.join(HERE, "inf_float_1k10k.json"), "w"))

        # integer 10k/100k, k=10, 8 queries (about 70 s each, run in parallel)
        ds = datagen.uniform(10_000, 100_000, seed=7, nq=8, k=10, integer=True)
        p = os.path.join(td, "int_big.txt")
        datagen.write_text(p, ds, integer=True)
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            futs = {int(q): ex.submit(run_ref, "rknn-naive-ids", p, int(q), 10) for q in ds.queries}
            res = {str(q): f.result()[0] for q, f in futs.items()}
        json.dump({"k": 10, "binary": "rknn-naive", "seed": 7, "nf": 10_000, "nu": 100_000,
                   "ids": res, "sha256": checksum(ds)},
                  open(os.path.join(HERE, "naive_int_10k100k.json"), "w"))

    json.dump(handmade(), open(os.path.join(HERE, "handmade.json"), "w"), indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
