"""CPU-side checks: the rknn-inf restatement against the reference binary's
own outputs, the exported C ABI, and the command line's argument handling."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import datagen
import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_inf_port_matches_reference_binary(golden_dir):
    """Over an 8-entry R-tree the port reproduces rknn-inf's bisector counts
    and result sets (golden vectors from the reference binary)."""
    g = json.load(open(os.path.join(golden_dir, "inf_float_1k10k.json")))
    z = np.load(os.path.join(golden_dir, "uniform_1k10k.npz"))
    port = O.InfPort(z["fxy"], z["uxy"], uid=z["uid"])
    for q, ids in g["ids"].items():
        bis, res, st = port.query(int(q), g["k"], skip_coincident=False)
        assert st["bisectors"] == g["bisectors"][q], q
        assert res.tolist() == ids, q


def test_inf_port_superset_of_exact():
    ds = datagen.uniform(500, 5000, seed=21, nq=20, k=4)
    port = O.InfPort(ds.fxy, ds.uxy, uid=ds.uid)
    o = O.Oracle.of(ds)
    for q in ds.queries:
        _, res, _ = port.query(int(q), 4)
        assert set(o.query(int(q), 4).tolist()) <= set(res.tolist())


def header_functions():
    txt = open(os.path.join(REPO, "include", "rknn_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rknn_[a-z_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(engine):
    names = header_functions()
    assert len(names) >= 10
    lib = engine.load()
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(engine.EXPORTS)
    assert b"sm_103a" in lib.rknn_version()


def test_fast_batch_entry_checks_its_buffers(engine):
    """The CPython entry point for rknn_query_batch (built where the
    interpreter's headers are installed) takes contiguous int32 buffers of
    equal length and hands anything else back as an argument error."""
    fast = engine._fast_call()
    if not fast:
        pytest.skip("no CPython headers here: the ctypes route is used")
    q = np.zeros(4, np.int32)
    assert fast.query_batch(0, q, np.ones(4, np.int32), 0, 0, 0, 0) == 1      # null index
    assert fast.query_batch(0, q, np.ones(3, np.int32), 0, 0, 0, 0) == 1      # lengths differ
    with pytest.raises((BufferError, ValueError)):       # not contiguous
        fast.query_batch(0, np.zeros(8, np.int32)[::2], np.ones(4, np.int32), 0, 0, 0, 0)


def test_cli_rejects_bad_arguments(engine, tmp_path):
    cli = os.path.join(REPO, "rt-rknn_gb300", "rknn-gb300")
    r = subprocess.run([cli, "-h"], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stderr
    r = subprocess.run([cli, "-if", str(tmp_path / "missing.txt"), "-k", "3"], capture_output=True, text=True)
    assert r.returncode == 1 and "Error opening file" in r.stderr
    r = subprocess.run([cli, "-if", "x", "-k", "0"], capture_output=True, text=True)
    assert r.returncode == 1 and "Invalid value for k" in r.stderr
    p = tmp_path / "bad.txt"
    p.write_text("2\n0 1 1\n1 2\n")
    r = subprocess.run([cli, "-if", str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and "Error parsing" in r.stderr


def test_snapshot_round_trip_and_checks(engine, tmp_path):
    """The binary snapshot (host code, no GPU): points written and read back
    bit for bit; a flipped byte or a cut file is refused; the command line's
    --save writes the same bytes as the library from the parsed text, and a
    snapshot given as -if loads the same points."""
    ds = datagen.uniform(300, 5000, seed=17)
    p = str(tmp_path / "pts.rkx")
    engine.snapshot_write(p, ds.fxy, ds.fid, ds.uxy, ds.uid)
    fxy, fid, uxy, uid = engine.snapshot_read(p)
    assert np.array_equal(fxy, ds.fxy) and np.array_equal(uxy, ds.uxy)
    assert np.array_equal(fid, ds.fid) and np.array_equal(uid, ds.uid)
    raw = bytearray(open(p, "rb").read())
    assert raw[:8] == b"RKNNSNP1" and len(raw) == 8 + 8 + 16 + 12 * ds.nf + 12 * ds.nu + 8
    bad = bytearray(raw)
    bad[40] ^= 1
    (tmp_path / "bad.rkx").write_bytes(bytes(bad))
    with pytest.raises(engine.RkNNError):
        engine.snapshot_read(str(tmp_path / "bad.rkx"))
    (tmp_path / "cut.rkx").write_bytes(bytes(raw[:-20]))
    with pytest.raises(engine.RkNNError):
        engine.snapshot_read(str(tmp_path / "cut.rkx"))
    # the command line: text in, --save out (it stops at the index build
    # when there is no GPU, after loading and saving)
    cli = os.path.join(REPO, "rt-rknn_gb300", "rknn-gb300")
    txt = tmp_path / "pts.txt"
    datagen.write_text(txt, ds)
    r = subprocess.run([cli, "-if", str(txt), "-k", "3", "--no-log", "--save", str(tmp_path / "cli.rkx")],
                       capture_output=True, text=True)
    assert f"Loaded {ds.nf} facilities and {ds.nu} users." in r.stdout
    assert open(tmp_path / "cli.rkx", "rb").read() == bytes(raw)
    r = subprocess.run([cli, "-if", p, "-k", "3", "--no-log"], capture_output=True, text=True)
    assert f"Loaded {ds.nf} facilities and {ds.nu} users." in r.stdout


def test_python_structs_match_the_header(engine, tmp_path):
    """Every public struct of include/rknn_gpu.h has the size and field
    offsets of its ctypes mirror in rknn.py (a C program built against the
    header prints them)."""
    import ctypes as C
    mirrors = {"rknn_index_opts": engine.Opts, "rknn_query_stats": engine.Stats, "rknn_index_info": engine.Info,
               "rknn_serve_opts": engine.ServeOpts, "rknn_serve_stats": engine.ServeStats,
               "rknn_tune_result": engine.TuneResult}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rknn_gpu.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", f"-I{os.path.join(REPO, 'include')}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_cli_parser_number_forms(engine, tmp_path):
    """The command line's text parser (from_chars, with strtoll/strtod for
    the forms from_chars does not take) reads ids and coordinates as the
    reference's stream extraction does: signs, exponents, a leading '+',
    hexadecimal floats, tabs and CR line ends; the points it saves as a
    snapshot equal Python's parse rounded to float32."""
    rows_f = [("0", "1.5", "2.25"), ("+1", "+3e2", "-4.5E-1"), ("2", "0x1.8p1", "7"), ("3", "1e-3", ".5")]
    rows_u = [("10", "0.1", "0.2"), ("11", "-0", "1e+1"), ("+12", "123456.789", "3.")]
    text = f"{len(rows_f)}\r\n" + "".join("\t".join(r) + "\r\n" for r in rows_f)
    text += f"{len(rows_u)}\n" + "".join(" ".join(r) + "\n" for r in rows_u)
    src = tmp_path / "forms.txt"
    src.write_text(text)
    cli = os.path.join(REPO, "rt-rknn_gb300", "rknn-gb300")
    snap = tmp_path / "forms.rkx"
    r = subprocess.run([cli, "-if", str(src), "-k", "1", "--no-log", "--save", str(snap)],
                       capture_output=True, text=True)
    assert "Loaded 4 facilities and 3 users." in r.stdout, r.stdout + r.stderr
    fxy, fid, uxy, uid = engine.snapshot_read(str(snap))

    def num(t):
        return float.fromhex(t) if "0x" in t else float(t)

    assert fid.tolist() == [int(r[0]) for r in rows_f] and uid.tolist() == [int(r[0]) for r in rows_u]
    assert np.array_equal(fxy, np.array([[num(r[1]), num(r[2])] for r in rows_f], np.float32))
    assert np.array_equal(uxy, np.array([[num(r[1]), num(r[2])] for r in rows_u], np.float32))


def _order_key(d):
    """order_key of rt-rknn_gb300/csrc/rknn_common.cuh restated: an int64
    key with the numeric order of finite doubles (-0 counts as +0)."""
    b = d.view(np.int64).copy()
    b[b == np.int64(-0x8000000000000000)] = 0
    return np.where(b >= 0, b, b ^ np.int64(0x7FFFFFFFFFFFFFFF))


def test_fp64_verification_bit_compares():
    """The small-batch FP64 verification decides mv < -bu and -bu <= mv <= bu
    on the bits (csrc/verify_item.cuh, filter_users with BITS): for finite mv
    and bu > 0, order_key(mv) < ~bits(bu) and |mv| <= bu on the magnitude
    bits.  Checked against the double compares on random values, signed
    zeros, subnormals, equal magnitudes and neighbours of bu."""
    rng = np.random.default_rng(7)
    n = 400_000
    bu = np.abs(rng.standard_normal(n)) * 10.0 ** rng.integers(-310, 300, n)
    bu = np.where(bu > 0, bu, 5e-324)
    mv = rng.standard_normal(n) * 10.0 ** rng.integers(-310, 300, n)
    pick = rng.integers(0, 8, n)
    mv = np.where(pick == 0, bu, mv)
    mv = np.where(pick == 1, -bu, mv)
    mv = np.where(pick == 2, np.nextafter(-bu, 0), mv)
    mv = np.where(pick == 3, np.nextafter(-bu, -np.inf), mv)
    mv = np.where(pick == 4, np.nextafter(bu, np.inf), mv)
    mv = np.where(pick == 5, np.where(rng.integers(0, 2, n) == 1, 0.0, -0.0), mv)
    mv = np.where(pick == 6, rng.choice([5e-324, -5e-324, 2.2e-308, -2.2e-308], n), mv)
    assert np.all(np.isfinite(mv)) and np.all(bu > 0)
    bb = bu.view(np.int64)
    lt = _order_key(mv) < ~bb
    inband = (mv.view(np.int64) & np.int64(0x7FFFFFFFFFFFFFFF)) <= bb
    assert np.array_equal(lt, mv < -bu)
    assert np.array_equal(inband, (mv <= bu) & (mv >= -bu))
