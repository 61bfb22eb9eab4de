"""Generate the golden fixtures under tests/golden/ from the reference implementation itself.

Run where a checkout of the reference is available:

    python tests/golden/make_golden.py PATH_TO_REFERENCE [--cases NAME,NAME]
    PIBRONIC_REFERENCE=PATH_TO_REFERENCE python tests/golden/make_golden.py

With --cases only the named seeded cases are (re)run and merged into reference_runs.npz.

It (1) packs the reference's own known-answer data (tests/pimc/explicit_data/*) into
explicit_example.npz, and (2) imports the unmodified reference engine from a temporary copy
(stub modules stand in for matplotlib and `parse`, which the engine never calls), runs
block_compute_pm, block_compute, the learned-proposal data path and the estimators on seeded
synthetic models, and records the sampled q and every output into reference_runs.npz, with the
model files as JSON text.  It also records (3) result files the reference wrote and merged
(reference_result_files.npz), (4) a data set of result files and the *_thermo files the
reference's file-driven estimators wrote from it (reference_analysis_files.npz), and (5) the job
scripts' parameter string and what BoxDataPM made of it (reference_job_parameters.npz), and (6) the
learned-proposal training files (reference_training_files.npz), and packs (7) the sum-over-states
results the reference's test data sets carry (reference_sos_results.npz), and (8) the diagonal
models the reference derives from coupled ones (reference_derived_models.npz).  The
fixtures are small; the GPU machine never needs the reference.
"""
from __future__ import annotations

import glob
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from pibronic_gb300 import synthetic, vibronic_io  # noqa: E402


def import_reference(ref_root):
    tmp = tempfile.mkdtemp(prefix="pbr_ref_")
    stubs = os.path.join(tmp, "stubs")
    os.makedirs(os.path.join(stubs, "matplotlib"))
    with open(os.path.join(stubs, "matplotlib", "__init__.py"), "w") as fh:
        fh.write("def use(*a, **k):\n    pass\n")
    open(os.path.join(stubs, "matplotlib", "pyplot.py"), "w").close()
    with open(os.path.join(stubs, "parse.py"), "w") as fh:
        fh.write("def parse(*a, **k):\n    raise NotImplementedError\n"
                 "def search(*a, **k):\n    raise NotImplementedError\n"
                 "def compile(*a, **k):\n    raise NotImplementedError\n")
    shutil.copytree(os.path.join(ref_root, "pibronic"), os.path.join(tmp, "pibronic"))
    sys.path[:0] = [stubs, tmp]
    import warnings
    warnings.simplefilter("ignore")
    import pibronic.pimc.pimc as engine
    import pibronic.stats.stats as st
    import pibronic.stats.jackknife as jk
    import pibronic.data.file_structure as fs
    import pibronic.constants as const
    return engine, st, jk, fs, const, tmp


def explicit_example(ref_root):
    src = os.path.join(ref_root, "tests", "pimc", "explicit_data")
    out = {}
    for path in sorted(glob.glob(os.path.join(src, "*.npy"))):
        key = os.path.basename(path)[:-4].replace("(", "_").replace(")", "")
        out[key] = np.load(path)
    for name in ("coupled_model", "sampling_model"):
        with open(os.path.join(src, name + ".json")) as fh:
            out[name + "_json"] = np.array(fh.read())
    np.savez_compressed(os.path.join(HERE, "explicit_example.npz"), **out)
    return sorted(out)


def sos_results(ref_root):
    """The reference's test data sets (tests/test_models/data_set_{0,1}): the coupled and sampling
    model files with the sum-over-states thermodynamics its Julia toolkit wrote beside them
    (sos_B60.json, sos_B80.json: Z, E, Cv of the coupled, harmonic and sampling models at 300 K,
    and Z_sampling at beta +- dbeta)."""
    src = os.path.join(ref_root, "tests", "test_models")
    out = {}
    for path in sorted(glob.glob(os.path.join(src, "data_set_*", "**", "sos_B*.json"), recursive=True)):
        rel = os.path.relpath(path, src)
        pdir = os.path.dirname(path)
        model = "sampling_model.json" if "rho_" in rel else "coupled_model.json"
        with open(path) as fh:
            out[f"{rel}/sos"] = np.array(fh.read())
        with open(os.path.join(pdir, model)) as fh:
            out[f"{rel}/model"] = np.array(fh.read())
    np.savez_compressed(os.path.join(HERE, "reference_sos_results.npz"), **out)
    return sorted(out)


def derived_models(ref_root):
    """The reference's remove_coupling_from_model (vibronic_model_io.py:749-761) on its test data
    sets' coupled models and on two synthetic ones: input and output model files as text."""
    import pibronic.vibronic.vibronic_model_io as vio
    src = os.path.join(ref_root, "tests", "test_models")
    texts = {}
    for path in sorted(glob.glob(os.path.join(src, "data_set_*", "parameters", "coupled_model.json"))):
        with open(path) as fh:
            texts[os.path.relpath(path, src)] = fh.read()
    tmp = tempfile.mkdtemp(prefix="pbr_derived_")
    for name in ("odd", "cfg4"):
        case = CASES[name]
        model = synthetic.make_coupled_model(case["A"], case["N"], case["model_seed"],
                                             sd_offdiag=case.get("sd_offdiag", 0.05))
        path = os.path.join(tmp, name + ".json")
        vibronic_io.save_model_to_JSON(path, model)
        with open(path) as fh:
            texts[f"synthetic_{name}"] = fh.read()
    out = {}
    for i, (name, text) in enumerate(sorted(texts.items())):
        src_path, dst_path = os.path.join(tmp, f"in_{i}.json"), os.path.join(tmp, f"out_{i}.json")
        with open(src_path, "w") as fh:
            fh.write(text)
        vio.remove_coupling_from_model(src_path, dst_path)
        with open(dst_path) as fh:
            out[f"{name}/coupled"], out[f"{name}/diagonal"] = np.array(text), np.array(fh.read())
    shutil.rmtree(tmp, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "reference_derived_models.npz"), **out)
    return sorted(out)


def write_models(root, case):
    """Write the case's model files under root/data_set_0/{parameters,rho_0/parameters}."""
    vib_dir = os.path.join(root, "data_set_0", "parameters")
    rho_dir = os.path.join(root, "data_set_0", "rho_0", "parameters")
    os.makedirs(vib_dir, exist_ok=True)
    os.makedirs(rho_dir, exist_ok=True)
    if "vib_json" in case:
        vib_text, rho_text = case["vib_json"], case["rho_json"]
    else:
        if case.get("degenerate"):
            model = synthetic.make_near_degenerate_model(case["A"], case["N"], case["model_seed"],
                                                         eps=case["degenerate"])
        else:
            model = synthetic.make_coupled_model(case["A"], case["N"], case["model_seed"],
                                                 sd_offdiag=case.get("sd_offdiag", 0.05),
                                                 sd_quadratic=case.get("sd_quadratic", 0.002))
        if case.get("zero_diag_linear"):
            # equal state shifts keep V symmetric when each surface slot holds R - d_a
            # (the learned-proposal data path asserts that symmetry, pimc.py:1169)
            for a in range(case["A"]):
                model[vibronic_io.VMK.G1][:, a, a] = 0.0
        rho = synthetic.diagonal_of(model)
        extra = case.get("extra_rho_surfaces", 0)
        if extra:
            A, N = case["A"], case["N"]
            VMK = vibronic_io.VMK
            rho[VMK.A] = A + extra
            rho[VMK.E] = np.concatenate([rho[VMK.E], 0.3 + 0.1 * np.arange(extra)])
            rho[VMK.G1] = np.concatenate([rho[VMK.G1], 0.02 * np.ones((N, extra))], axis=1)
            rho[VMK.G2] = np.zeros((N, N, A + extra))
        vibronic_io.save_model_to_JSON(os.path.join(vib_dir, "coupled_model.json"), model)
        vibronic_io.save_diagonal_model_to_JSON(os.path.join(rho_dir, "sampling_model.json"), rho)
        with open(os.path.join(vib_dir, "coupled_model.json")) as fh:
            vib_text = fh.read()
        with open(os.path.join(rho_dir, "sampling_model.json")) as fh:
            rho_text = fh.read()
    with open(os.path.join(vib_dir, "coupled_model.json"), "w") as fh:
        fh.write(vib_text)
    with open(os.path.join(rho_dir, "sampling_model.json"), "w") as fh:
        fh.write(rho_text)
    return vib_text, rho_text


def run_case(engine, fs, const, case, files=None):
    """Run block_compute(_pm) of the reference on the case; with `files` (a dict), also keep the
    result file the run wrote (pimc.py:1383, 1461) and two the reference's BoxResult writes and
    merges around it (pimc.py:819-835, 948-964, 853-912, 975-1040)."""
    root = tempfile.mkdtemp(prefix="pbr_case_")
    vib_text, rho_text = write_models(root, case)
    FS = fs.FileStructure(root, 0, 0)
    FS.generate_model_hashes()
    pm = case.get("pm", True)
    beta = const.beta(case["T"])
    data = engine.BoxDataPM(case.get("dbeta_rel", 1e-4) * beta) if pm else engine.BoxData()
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.hash_vib, data.hash_rho = FS.hash_vib, FS.hash_rho
    A, N = json.loads(vib_text)["number of surfaces"], json.loads(vib_text)["number of modes"]
    data.states, data.modes = A, N
    data.samples, data.beads, data.temperature = case["X"], case["P"], case["T"]
    data.block_size = case["B"]
    data.blocks = data.samples // data.block_size
    np.random.seed(case["rng_seed"])
    recorded = []
    original = engine.BoxData.transform_sampled_coordinates

    def recording(self, sample_view):
        original(self, sample_view)
        recorded.append(self.qTensor[:, 0].copy())

    engine.BoxData.transform_sampled_coordinates = recording
    try:
        import contextlib
        import io
        with contextlib.redirect_stdout(io.StringIO()):
            data.preprocess()
            result = engine.BoxResultPM(data=data) if pm else engine.BoxResult(data=data)
            result.path_root = FS.path_rho_results
            result.id_job = 0
            (engine.block_compute_pm if pm else engine.block_compute)(data, result)
    finally:
        engine.BoxData.transform_sampled_coordinates = original
    out = {"q": np.concatenate(recorded), "s_rho": result.scaled_rho.copy(),
           "s_g": result.scaled_g.copy(), "beta": beta, "tau": data.tau,
           "delta_beta": data.delta_beta if pm else 0.0,
           "state_weight": data.rho.state_weight.copy(),
           "sample_sources": data.rho.sample_sources.copy(),
           "vib_json": np.array(vib_text), "rho_json": np.array(rho_text)}
    if pm:
        out["s_gP"] = result.scaled_gofr_plus.copy()
        out["s_gM"] = result.scaled_gofr_minus.copy()
    if files is not None:
        keep_result_files(engine, FS, data, result, pm, files)
    shutil.rmtree(root, ignore_errors=True)
    return out


def keep_result_files(engine, FS, data, result, pm, files):
    """The run's own file (J0), a second job's file written by the reference from doubled arrays
    (J1), a file of the other result class (J2: its keys are a subset or a superset), and the
    reference's merge of the three; merge order follows a Python set, so the merged arrays are
    recorded sorted by s_rho."""
    cls = engine.BoxResultPM if pm else engine.BoxResult
    other = engine.BoxResult if pm else engine.BoxResultPM
    path0 = result.compute_path_to_file()
    second = cls(data=data)
    second.path_root, second.id_job = result.path_root, 1
    second.scaled_rho, second.scaled_g = 2.0 * result.scaled_rho, 2.0 * result.scaled_g
    if pm:
        second.scaled_gofr_plus = 2.0 * result.scaled_gofr_plus
        second.scaled_gofr_minus = 2.0 * result.scaled_gofr_minus
    second.save_results(data.samples)
    path1 = second.compute_path_to_file()
    third = other(data=data)
    third.path_root, third.id_job = result.path_root, 2
    third.scaled_rho, third.scaled_g = 3.0 * result.scaled_rho, 3.0 * result.scaled_g
    if not pm:
        third.scaled_gofr_plus = 3.0 * result.scaled_rho
        third.scaled_gofr_minus = 3.0 * result.scaled_g
    third.save_results(data.samples)
    path2 = third.compute_path_to_file()
    for j, path in enumerate((path0, path1, path2)):
        files[f"name_J{j}"] = np.array(os.path.basename(path))
        with open(path, "rb") as fh:
            files[f"bytes_J{j}"] = np.frombuffer(fh.read(), dtype=np.uint8)
    merged = cls()
    merged.load_multiple_results([path0, path1, path2])
    order = np.argsort(merged.scaled_rho, kind="stable")
    files["merged_samples"] = np.int64(merged.samples)
    files["merged_s_rho"] = np.asarray(merged.scaled_rho)[order]
    files["merged_s_g"] = np.asarray(merged.scaled_g)[order]
    if pm:
        files["merged_s_gP"] = np.asarray(merged.scaled_gofr_plus)[order]
        files["merged_s_gM"] = np.asarray(merged.scaled_gofr_minus)[order]
    files["P"], files["T"] = np.int64(data.beads), np.float64(data.temperature)
    files["hash_vib"], files["hash_rho"] = np.array(data.hash_vib), np.array(data.hash_rho)


ANALYSIS_JOBS = [  # (P, T, J, X, rng_seed, beta +- dbeta) on the full (P, T) grid the reference
    # analyses (every pair must have a file): two jobs at one pair, a plain run beside another
    (12, 300.0, 0, 40, 501, True), (12, 300.0, 1, 40, 502, True), (12, 250.0, 0, 20, 503, True),
    (8, 300.0, 0, 20, 504, True), (8, 250.0, 0, 30, 505, True), (8, 250.0, 1, 30, 506, False)]


def analysis_files(engine, st, fs, const):
    """A data set with result files from several jobs and an analytic-results file, and the
    *_thermo files the reference's file-driven estimators write from it
    (stats.py:148-179, 219-265, 336-377) for each method, basic and alpha, with and without the
    jackknife.  The analytic file is the package's closed form in the reference's layout (the
    reference takes it from its Julia toolkit); the estimators only read it."""
    from pibronic_gb300 import analytic
    from pibronic_gb300 import file_structure as our_fs
    import contextlib
    import io
    root = tempfile.mkdtemp(prefix="pbr_stats_")
    case = dict(CASES["cfg1"])
    vib_text, rho_text = write_models(root, case)
    FS = fs.FileStructure(root, 0, 0)
    FS.generate_model_hashes()
    A = json.loads(vib_text)["number of surfaces"]
    N = json.loads(vib_text)["number of modes"]
    out = {"vib_json": np.array(vib_text), "rho_json": np.array(rho_text)}
    with contextlib.redirect_stdout(io.StringIO()):
        for P, T, J, X, seed, pm in ANALYSIS_JOBS:
            data = engine.BoxDataPM(const.delta_beta) if pm else engine.BoxData()
            data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
            data.hash_vib, data.hash_rho = FS.hash_vib, FS.hash_rho
            data.states, data.modes = A, N
            data.samples, data.beads, data.temperature = X, P, T
            data.block_size = X // 2
            data.blocks = 2
            np.random.seed(seed)
            data.preprocess()
            result = engine.BoxResultPM(data=data) if pm else engine.BoxResult(data=data)
            result.path_root, result.id_job = FS.path_rho_results, J
            (engine.block_compute_pm if pm else engine.block_compute)(data, result)
        ours = our_fs.FileStructure(root, 0, 0)
        for T in sorted({job[1] for job in ANALYSIS_JOBS}):
            analytic.analytic_of_sampling_model(ours, const.beta(T))
        for path in sorted(glob.glob(os.path.join(FS.path_rho_results, "*.npz"))):
            name = os.path.basename(path)
            with open(path, "rb") as fh:
                out[f"result/{name}"] = np.frombuffer(fh.read(), dtype=np.uint8)
        with open(FS.path_analytic_rho) as fh:
            out["analytic_json"] = np.array(fh.read())
        for method in ("basic", "alpha"):
            for tag, driver in (("stats", st.statistical_analysis_of_pimc),
                                ("jk", st.jackknife_analysis_of_pimc)):
                for path in glob.glob(os.path.join(FS.path_rho_results, "*_thermo")):
                    os.remove(path)
                driver(FS, method=method)
                for path in sorted(glob.glob(os.path.join(FS.path_rho_results, "*_thermo"))):
                    with open(path) as fh:
                        out[f"thermo/{tag}_{method}/{os.path.basename(path)}"] = np.array(fh.read())
    np.savez_compressed(os.path.join(HERE, "reference_analysis_files.npz"), **out)
    shutil.rmtree(root, ignore_errors=True)
    return sorted(out)


def job_parameters(engine, fs, const):
    """The job scripts' sequence up to the block loop (server/compute_canada/pimc.py:20-36): a
    parameter dict as the job submitter builds it (server/job_boss.py:415-470), serialised by the
    reference's BoxData.json_serialize, read back by BoxDataPM.from_json_string, preprocess, and
    the result file name of job "3".  The data set root is recorded as the token @ROOT@."""
    import contextlib
    import io
    root = tempfile.mkdtemp(prefix="pbr_job_")
    D, R = 2, 1
    case = dict(CASES["odd"])
    vib_dir = os.path.join(root, f"data_set_{D}", "parameters")
    rho_dir = os.path.join(root, f"data_set_{D}", f"rho_{R}", "parameters")
    tmp_case = tempfile.mkdtemp(prefix="pbr_jobm_")
    vib_text, rho_text = write_models(tmp_case, case)
    shutil.rmtree(tmp_case, ignore_errors=True)
    os.makedirs(vib_dir)
    os.makedirs(rho_dir)
    with open(os.path.join(vib_dir, "coupled_model.json"), "w") as fh:
        fh.write(vib_text)
    with open(os.path.join(rho_dir, "sampling_model.json"), "w") as fh:
        fh.write(rho_text)
    params = {"number_of_samples": 40, "number_of_blocks": 4, "number_of_states": case["A"],
              "number_of_modes": case["N"], "number_of_beads": case["P"], "temperature": case["T"],
              "block_size": 10, "delta_beta": 2e-4, "id_data": D, "id_rho": R, "path_root": root,
              "path_scratch": os.path.join(root, f"data_set_{D}", f"rho_{R}") + "/",
              "hostname": "node", "partition": None}
    text = engine.BoxData.json_serialize(params)
    out = {"json": np.array(text.replace(root, "@ROOT@")), "vib_json": np.array(vib_text),
           "rho_json": np.array(rho_text)}
    with contextlib.redirect_stdout(io.StringIO()):
        data = engine.BoxDataPM.from_json_string(text)
        fields = {k: getattr(data, k) for k in ("samples", "blocks", "states", "beads", "modes",
                                                 "temperature", "block_size", "id_data", "id_rho",
                                                 "beta", "tau", "delta_beta", "hash_vib", "hash_rho")}
        data.preprocess()
        fields.update({k + "_pre": getattr(data, k) for k in ("beta", "tau", "beta_plus", "beta_minus",
                                                              "tau_plus", "tau_minus")})
        FS = fs.FileStructure.from_boxdata(os.path.normpath(os.path.join(params["path_scratch"], "../..")), data)
        result = engine.BoxResultPM(data=data)
        result.path_root, result.id_job = FS.path_rho_results, "3"
        fields["result_path"] = result.compute_path_to_file().replace(root, "@ROOT@")
    for k, v in fields.items():
        out[f"field/{k}"] = np.array(v)
    np.savez_compressed(os.path.join(HERE, "reference_job_parameters.npz"), **out)
    shutil.rmtree(root, ignore_errors=True)
    return sorted(out)


def result_files(engine, fs, const):
    """Result files of a beta +- dbeta run (cfg1 shapes) and of a plain run (the `plain` case)."""
    out = {}
    for tag, name in (("pm", "cfg1"), ("plain", "plain")):
        files = {}
        run_case(engine, fs, const, dict(CASES[name], X=12, B=6), files=files)
        for k, v in files.items():
            out[f"{tag}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "reference_result_files.npz"), **out)
    return sorted(out)


ML_CASE = dict(A=2, N=3, P=8, T=300.0, X=30, B=15, model_seed=17, rng_seed=2024, zero_diag_linear=True)


def run_ml_case(engine, fs, case, files=None):
    """block_compute_gR_from_raw_samples + block_compute_rhoR_from_input_samples; with `files`
    (a dict), also keep the training files the first wrote (pimc.py:1250-1270, 1305-1338)."""
    root = tempfile.mkdtemp(prefix="pbr_ml_")
    vib_text, rho_text = write_models(root, case)
    FS = fs.FileStructure(root, 0, 0)
    FS.generate_model_hashes()
    data = engine.BoxData.from_FileStructure(FS)
    data.hash_vib, data.hash_rho = FS.hash_vib, FS.hash_rho
    data.samples, data.beads, data.temperature = case["X"], case["P"], case["T"]
    data.block_size = case["B"]
    data.blocks = data.samples // data.block_size
    np.random.seed(case["rng_seed"])
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        data.preprocess()
        result = engine.BoxResult(data=data)
        result.id_job = 0
        result.path_root = FS.path_vib_results
        engine.block_compute_gR_from_raw_samples(data, result)
        g = result.scaled_g.copy()
        with np.load(os.path.join(FS.path_vib_results,
                                  f"P{case['P']}_T{case['T']:.2f}_J0_training_data_input.npz")) as d:
            R = d["input_R_values"].copy()
        res2 = engine.BoxResult(data=data)
        engine.block_compute_rhoR_from_input_samples(data, res2, R)
    if files is not None:
        for path in sorted(glob.glob(os.path.join(FS.path_vib_results, "*_training_data_*.npz"))):
            with open(path, "rb") as fh:
                files[os.path.basename(path)] = np.frombuffer(fh.read(), dtype=np.uint8)
        files["P"], files["T"], files["X"] = np.int64(case["P"]), np.float64(case["T"]), np.int64(case["X"])
    shutil.rmtree(root, ignore_errors=True)
    return {"R": R, "g": g, "rho": res2.scaled_rho.copy(), "vib_json": np.array(vib_text),
            "rho_json": np.array(rho_text)}


CASES = {
    # the smallest benchmark shapes: A=2, N=2, P=12, T=300 K, quadratic terms, dbeta = 1e-4 beta
    "cfg1": dict(A=2, N=2, P=12, T=300.0, X=400, B=100, model_seed=11, rng_seed=1234),
    # the main benchmark shapes at a small sample count: A=4, N=12, P=64
    "cfg2": dict(A=4, N=12, P=64, T=300.0, X=60, B=20, model_seed=22, rng_seed=4321),
    # the same shapes at the low temperature of their sweep
    "cfg2_cold": dict(A=4, N=12, P=64, T=100.0, X=40, B=20, model_seed=23, rng_seed=99),
    # odd bead count, three surfaces, strong off-diagonal couplings
    "odd": dict(A=3, N=5, P=7, T=250.0, X=50, B=25, model_seed=5, rng_seed=77, sd_offdiag=0.1),
    # plain block_compute (no beta +- db)
    "plain": dict(A=2, N=3, P=16, T=300.0, X=50, B=25, model_seed=8, rng_seed=31, pm=False),
    # sampling model with more surfaces than the coupled model (qTempTensor path)
    "arho": dict(A=2, N=3, P=10, T=300.0, X=60, B=30, model_seed=9, rng_seed=55, extra_rho_surfaces=2),
    # one surface
    "single_surface": dict(A=1, N=4, P=8, T=300.0, X=40, B=20, model_seed=3, rng_seed=8),
    # learned-proposal configuration shapes: A=6, N=20, P=128, T=200 K, strong off-diagonal couplings
    "cfg4": dict(A=6, N=20, P=128, T=200.0, X=16, B=8, model_seed=44, rng_seed=404, sd_offdiag=0.1),
    # the largest surface count of the batched configuration
    "a8": dict(A=8, N=5, P=16, T=400.0, X=24, B=12, model_seed=88, rng_seed=808),
    # seven surfaces, odd everything
    "a7": dict(A=7, N=3, P=9, T=150.0, X=21, B=7, model_seed=77, rng_seed=707),
    # more surfaces than the row-team form holds (the tensor-core and wide forms): 12 and 16
    "a12": dict(A=12, N=4, P=8, T=300.0, X=12, B=6, model_seed=1212, rng_seed=1213),
    "a16": dict(A=16, N=3, P=6, T=250.0, X=8, B=4, model_seed=1616, rng_seed=1617),
    # the smallest ring the reference accepts (3 beads) with a single mode
    "p3_n1": dict(A=2, N=1, P=3, T=500.0, X=30, B=10, model_seed=31, rng_seed=313),
    # hot (1000 K, short tau) and cold (50 K, long tau) ends of the temperature range
    "hot": dict(A=3, N=4, P=16, T=1000.0, X=30, B=15, model_seed=1000, rng_seed=1001),
    "frozen": dict(A=2, N=3, P=32, T=50.0, X=20, B=10, model_seed=50, rng_seed=51),
    # the main benchmark shapes at the high temperature of their sweep (500 K)
    "cfg2_hot": dict(A=4, N=12, P=64, T=500.0, X=40, B=20, model_seed=25, rng_seed=505),
    # near-degenerate surfaces: equal diagonal terms, off-diagonal couplings ~ 1e-7 eV (two
    # surfaces: the Jacobi rotation; four: the scaling-and-squaring exponential; seven: the
    # row-team form's Jacobi; twelve: the wide form on the tensor-core potential)
    "degen2": dict(A=2, N=3, P=16, T=300.0, X=30, B=15, model_seed=72, rng_seed=721, degenerate=1e-7),
    "degen4": dict(A=4, N=6, P=32, T=300.0, X=30, B=15, model_seed=74, rng_seed=741, degenerate=1e-7),
    "degen7": dict(A=7, N=3, P=8, T=300.0, X=21, B=7, model_seed=77, rng_seed=771, degenerate=1e-7),
    "degen12": dict(A=12, N=4, P=8, T=300.0, X=12, B=6, model_seed=712, rng_seed=7121, degenerate=1e-7),
}


def add_cases(ref_root, names):
    """Run only the named CASES through the reference and merge them into reference_runs.npz
    (every other fixture and entry is left as it is)."""
    engine, st, jk, fs, const, tmp = import_reference(ref_root)
    path = os.path.join(HERE, "reference_runs.npz")
    with np.load(path) as d:
        runs = {k: d[k] for k in d.files}
    for name in names:
        runs = {k: v for k, v in runs.items() if not k.startswith(name + "/")}
        out = run_case(engine, fs, const, CASES[name])
        for k, v in out.items():
            runs[f"{name}/{k}"] = v
        print(name, {k: np.shape(v) for k, v in out.items()})
    np.savez_compressed(path, **runs)
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(CASES, fh, indent=1)
    shutil.rmtree(tmp, ignore_errors=True)


def main(ref_root):
    keys = explicit_example(ref_root)
    print("explicit_example.npz:", keys)
    print("reference_sos_results.npz:", sos_results(ref_root))
    engine, st, jk, fs, const, tmp = import_reference(ref_root)
    runs = {}
    for name, case in CASES.items():
        out = run_case(engine, fs, const, case)
        for k, v in out.items():
            runs[f"{name}/{k}"] = v
        print(name, {k: np.shape(v) for k, v in out.items()})
    # reference test models (tests/test_models/data_set_1/rho_1), block_compute_pm
    with open(os.path.join(ref_root, "tests/test_models/data_set_1/parameters/coupled_model.json")) as fh:
        vt = fh.read()
    with open(os.path.join(ref_root, "tests/test_models/data_set_1/rho_1/parameters/sampling_model.json")) as fh:
        rt = fh.read()
    out = run_case(engine, fs, const, dict(vib_json=vt, rho_json=rt, P=12, T=300.0, X=40, B=20,
                                            rng_seed=242351, dbeta_rel=const.delta_beta / const.beta(300.0)))
    for k, v in out.items():
        runs[f"testmodel/{k}"] = v
    # estimators on the cfg1 run (stats.py:38-130, jackknife.py:60-105)
    c = {k.split("/")[1]: v for k, v in runs.items() if k.startswith("cfg1/")}
    X, T, dB = len(c["s_rho"]), 300.0, float(c["delta_beta"])
    terms = st.calculate_basic_property_terms(dB, c["s_rho"], c["s_g"], c["s_gP"], c["s_gM"])
    basic = st.estimate_basic_properties(X, T, *terms)
    jkt = jk.calculate_jackknife_terms(X, terms)
    jkd = jk.estimate_jackknife(X, T, dB, basic, *jkt)
    for k, v in basic.items():
        runs[f"stats/basic/{k}"] = np.float64(v)
    for k, v in jkd.items():
        runs[f"stats/jk/{k}"] = np.float64(v)
    # learned-proposal data path
    training = {}
    ml = run_ml_case(engine, fs, ML_CASE, files=training)
    for k, v in ml.items():
        runs[f"ml/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "reference_training_files.npz"), **training)
    np.savez_compressed(os.path.join(HERE, "reference_runs.npz"), **runs)
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(CASES, fh, indent=1)
    print("reference_result_files.npz:", result_files(engine, fs, const))
    print("reference_analysis_files.npz:", analysis_files(engine, st, fs, const))
    print("reference_job_parameters.npz:", job_parameters(engine, fs, const))
    print("reference_derived_models.npz:", derived_models(ref_root))
    shutil.rmtree(tmp, ignore_errors=True)
    print("wrote", os.path.join(HERE, "reference_runs.npz"))


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("reference", nargs="?", default=os.environ.get("PIBRONIC_REFERENCE"),
                    help="root of the reference checkout (or set PIBRONIC_REFERENCE)")
    ap.add_argument("--cases", default="", help="comma-separated CASES to (re)run and merge into "
                    "reference_runs.npz, leaving every other fixture as it is")
    a = ap.parse_args()
    if not a.reference:
        ap.error("give the reference checkout's root (argument or PIBRONIC_REFERENCE)")
    if a.cases:
        add_cases(a.reference, [c for c in a.cases.split(",") if c])
    else:
        main(a.reference)
