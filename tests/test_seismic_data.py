"""SeismicData npz format parity with the reference (ADFWI/survey/data.py:63-99), on the CPU.

Fixtures written by the reference itself (``tests/golden/make_golden.py``):
``seismicdata_ref.npz`` is a file its ``SeismicData.save`` wrote; ``seismicdata_ours_read_by_ref.npz``
holds what its ``SeismicData.load`` read from a file this package's ``save`` wrote. Both come from
the seeded survey and records of ``tests/golden/seismic_case.py``.
"""
import os
import sys

import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from _cases import GOLDEN

sys.path.insert(0, GOLDEN)
from seismic_case import seismic_data_case  # noqa: E402

META = ("src_loc", "rcv_loc", "src_num", "rcv_num", "rcv_type", "src_type", "t", "nt", "dt")


def _ours():
    sv, recs = seismic_data_case(A.Source, A.Receiver, A.Survey, A.wavelet)
    d = A.SeismicData(sv)
    d.record_data({k: torch.tensor(v) for k, v in recs.items()})
    return sv, recs, d


def test_reference_written_file_loads_identically():
    sv, recs, _ = _ours()
    d = A.SeismicData(sv)
    d.load(os.path.join(GOLDEN, "seismicdata_ref.npz"))
    assert sorted(d.data) == sorted(recs)
    for k, v in recs.items():
        assert d.data[k].dtype == v.dtype and np.array_equal(d.data[k], v), k
    mine = A.SeismicData(sv)
    for k in META:
        assert np.array_equal(np.asarray(getattr(d, k)), np.asarray(getattr(mine, k))), k


def test_our_file_has_the_reference_layout(tmp_path):
    """Key for key, the file our save writes holds the same arrays (dtype, shape, values) as the
    one the reference's save wrote from the same survey and records."""
    _, _, d = _ours()
    path = str(tmp_path / "ours.npz")
    d.save(path)
    ours = np.load(path, allow_pickle=True)
    ref = np.load(os.path.join(GOLDEN, "seismicdata_ref.npz"), allow_pickle=True)
    assert sorted(ours.files) == sorted(ref.files)
    for k in ref.files:
        a, b = ours[k], ref[k]
        if k == "data":
            a, b = a.item(), b.item()
            assert sorted(a) == sorted(b)
            for c in b:
                assert a[c].dtype == b[c].dtype and np.array_equal(a[c], b[c]), c
        else:
            assert a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a, b), k


def test_reference_load_read_our_file():
    """What the reference's load read from a file our save wrote (recorded by make_golden.py)."""
    sv, recs, _ = _ours()
    g = np.load(os.path.join(GOLDEN, "seismicdata_ours_read_by_ref.npz"), allow_pickle=True)
    for k, v in recs.items():
        assert np.array_equal(g["data_" + k], v), k
    mine = A.SeismicData(sv)
    for k in META:
        assert np.array_equal(g[k], np.asarray(getattr(mine, k))), k


def test_parse_methods_follow_the_reference():
    _, recs, d = _ours()
    d.data["tzz"] = d.data["txx"][::-1].copy()
    d.data["txz"] = d.data["vx"] * 0.5
    d.data["vz"] = d.data["u"] - 1.0
    p, txz, vx, vz = d.parse_elastic_data(normalize=True)
    pr = -(d.data["txx"] + d.data["tzz"])
    assert np.array_equal(p, pr / np.max(np.abs(pr), axis=1, keepdims=True))
    assert np.array_equal(vz, d.data["vz"] / np.max(np.abs(d.data["vz"]), axis=1, keepdims=True))
    pa, ua, wa = d.parse_acoustic_data(normalize=False)
    assert pa is d.data["p"] and ua is d.data["u"] and wa is d.data["w"]


def test_reference_load_on_our_file_when_the_reference_is_present(tmp_path):
    """Live check in a container that holds the reference (skipped elsewhere): the reference's
    load, run in a child process by make_golden.py, reads back the records our save wrote."""
    import json
    import subprocess
    ref_root = os.environ.get("ADFWI_REFERENCE", "/root/reference")
    if not os.path.isdir(os.path.join(ref_root, "ADFWI")):
        pytest.skip("reference not present")
    _, recs, d = _ours()
    path = str(tmp_path / "ours.npz")
    d.save(path)
    r = subprocess.run([sys.executable, os.path.join(GOLDEN, "make_golden.py"), "--ref", ref_root,
                        "--read-with-reference", path], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, PYTHONDONTWRITEBYTECODE="1"))
    assert r.returncode == 0, r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    for k, v in recs.items():
        assert got["data"][k] == [list(v.shape), str(v.dtype), float(np.float64(v).sum()),
                                  float(np.abs(np.float64(v)).sum())], k
