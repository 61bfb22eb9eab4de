"""BoxResult / BoxResultPM ``.npz`` files against files the reference itself wrote and merged
(tests/golden/make_golden.py: pimc.py:819-835 and 948-964 write, 853-912 and 975-1040 merge).

Host logic only: no device is touched."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import GOLDEN
from pibronic_gb300 import pimc

KEYS = {"pm": ["hash_vib", "hash_rho", "number_of_samples", "s_rho", "s_g", "s_gP", "s_gM"],
        "plain": ["hash_vib", "hash_rho", "number_of_samples", "s_rho", "s_g"]}
CLS = {"pm": pimc.BoxResultPM, "plain": pimc.BoxResult}


@pytest.fixture(scope="module")
def ref_files():
    with np.load(os.path.join(GOLDEN, "reference_result_files.npz")) as d:
        return {k: d[k] for k in d.files}


def _unpack(ref_files, tag, root):
    paths = []
    for j in range(3):
        path = os.path.join(root, str(ref_files[f"{tag}/name_J{j}"]))
        with open(path, "wb") as fh:
            fh.write(ref_files[f"{tag}/bytes_J{j}"].tobytes())
        paths.append(path)
    return paths


def _arrays(res, tag):
    out = {"s_rho": res.scaled_rho, "s_g": res.scaled_g}
    if tag == "pm":
        out.update(s_gP=res.scaled_gofr_plus, s_gM=res.scaled_gofr_minus)
    return out


@pytest.mark.parametrize("tag", ["pm", "plain"])
def test_reads_a_reference_result_file(ref_files, tag, tmp_path):
    path = _unpack(ref_files, tag, str(tmp_path))[0]
    res = CLS[tag]()
    res.load_results(path)
    with np.load(path) as d:
        assert res.samples == int(d["number_of_samples"])
        for k, v in _arrays(res, tag).items():
            assert np.array_equal(v, d[k]), k


@pytest.mark.parametrize("tag", ["pm", "plain"])
def test_writes_the_reference_file_name_keys_and_types(ref_files, tag, tmp_path):
    (tmp_path / "ref").mkdir()
    ref_path = _unpack(ref_files, tag, str(tmp_path / "ref"))[0]
    data = SimpleNamespace(beads=int(ref_files[f"{tag}/P"]), temperature=float(ref_files[f"{tag}/T"]),
                           samples=0, hash_vib=str(ref_files[f"{tag}/hash_vib"]),
                           hash_rho=str(ref_files[f"{tag}/hash_rho"]))
    with np.load(ref_path) as ref:
        data.samples = int(ref["number_of_samples"])
        res = CLS[tag](data=data)
        res.path_root, res.id_job = str(tmp_path), 0
        res.scaled_rho, res.scaled_g = ref["s_rho"].copy(), ref["s_g"].copy()
        if tag == "pm":
            res.scaled_gofr_plus, res.scaled_gofr_minus = ref["s_gP"].copy(), ref["s_gM"].copy()
        res.save_results(data.samples)
        mine = res.compute_path_to_file()
        assert os.path.basename(mine) == str(ref_files[f"{tag}/name_J0"])
        with np.load(mine) as d:
            assert sorted(d.files) == sorted(ref.files) == sorted(KEYS[tag])
            for k in ref.files:
                assert d[k].dtype == ref[k].dtype and d[k].shape == ref[k].shape, k
                assert np.array_equal(d[k], ref[k]), k


@pytest.mark.parametrize("tag", ["pm", "plain"])
def test_merges_result_files_like_the_reference(ref_files, tag, tmp_path):
    """J0 and J1 share the class; J2 is the other class: a beta +- dbeta merge skips a plain file,
    a plain merge takes a beta +- dbeta file.  The reference's merge order follows a Python set,
    so the arrays are compared sorted by s_rho."""
    paths = _unpack(ref_files, tag, str(tmp_path))
    res = CLS[tag]()
    res.load_multiple_results(paths)
    assert res.samples == int(ref_files[f"{tag}/merged_samples"])
    order = np.argsort(res.scaled_rho, kind="stable")
    for k, v in _arrays(res, tag).items():
        assert np.array_equal(v[order], ref_files[f"{tag}/merged_{k}"]), k


@pytest.mark.parametrize("tag", ["pm", "plain"])
def test_merge_truncates_to_the_requested_count(ref_files, tag, tmp_path):
    paths = _unpack(ref_files, tag, str(tmp_path))
    n0 = int(np.load(paths[0])["number_of_samples"])
    res = CLS[tag]()
    res.load_multiple_results(paths, desired_number_of_samples=n0 + 3)
    assert res.samples == n0 + 3
    for v in _arrays(res, tag).values():
        assert not np.any(np.isnan(v))


def test_merge_rejects_lists_without_a_complete_file(ref_files, tmp_path):
    plain_path = _unpack(ref_files, "plain", str(tmp_path))[0]
    with pytest.raises(AssertionError):
        pimc.BoxResultPM().load_multiple_results([plain_path])
    with pytest.raises(AssertionError):
        pimc.BoxResultPM().load_multiple_results([])


def test_load_rejects_a_file_of_another_sample_count(ref_files, tmp_path):
    path = _unpack(ref_files, "pm", str(tmp_path))[0]
    res = pimc.BoxResultPM(X=5)
    with pytest.raises(AssertionError):
        res.load_results(path)


def test_training_files_match_the_reference(tmp_path):
    """save_gR_with_samples (pimc.py:1250-1270) against the training files the reference's
    block_compute_gR_from_raw_samples wrote: same names, keys, dtypes and values."""
    with np.load(os.path.join(GOLDEN, "reference_training_files.npz")) as f:
        ref = {k: f[k] for k in f.files}
    names = sorted(k for k in ref if k.endswith(".npz"))
    (tmp_path / "ref").mkdir()
    loaded = {}
    for name in names:
        path = tmp_path / "ref" / name
        path.write_bytes(ref[name].tobytes())
        with np.load(path) as d:
            loaded[name] = {k: d[k] for k in d.files}
    g_name = next(n for n in names if n.endswith("_g_output.npz"))
    in_name = next(n for n in names if n.endswith("_input.npz"))
    data = SimpleNamespace(beads=int(ref["P"]), temperature=float(ref["T"]), samples=int(ref["X"]),
                           hash_vib="v", hash_rho="r")
    res = pimc.BoxResult(data=data)
    res.path_root, res.id_job = str(tmp_path), 0
    res.scaled_g = loaded[g_name]["g"].copy()
    pimc.save_gR_with_samples(data, res, loaded[in_name]["input_R_values"])
    for name in names:
        with np.load(tmp_path / name) as d:
            assert sorted(d.files) == sorted(loaded[name]), name
            for k, v in loaded[name].items():
                assert d[k].dtype == v.dtype and np.array_equal(d[k], v), (name, k)
