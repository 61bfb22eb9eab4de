"""Drop-in replacement for Pibronic's PIMC engine ``pibronic.pimc`` (pibronic/pimc/pimc.py, the module
the reference README calls ``pimc/minimal.py``) running on one GB300.

Same public names, arguments, result arrays, ``.npz`` result files and error types:
``BoxData``/``BoxDataPM``, ``BoxResult``/``BoxResultPM``, ``block_compute``, ``block_compute_pm``,
the stage functions ``build_o_matrix``, ``build_scaling_factors``, ``scale_o_matrices``,
``build_denominator``, ``diagonalize_coupling_matrix``, ``build_numerator`` and the learned-proposal
data path ``block_compute_gR*`` / ``block_compute_rhoR_from_input_samples``.

``block_compute(_pm)`` run the fused CUDA kernel (``pbr_sample_eval``) over all samples; the stage
functions run the FP64 stage kernels on device tensors.  There is no CPU fallback: without the
CUDA library or a device the calls raise.

Differences a caller can see: samples come from a counter-based Philox stream keyed by
``data.seed`` (drawn from numpy's global generator in ``preprocess``, so ``np.random.seed``
still makes runs reproducible) instead of numpy's MT19937, and the sample sources are drawn per
sample on the device instead of all X up front (pimc.py:386-394, which also printed them).
"""
from __future__ import annotations

import json
import os
from functools import partial

import numpy as np

from . import _native
from . import constants
from . import file_structure as file_structure
from . import vibronic_io as vIO
from .plan import DevicePlan, PreparedModels, ring_mode_basis
from .vibronic_io import VMK

F64 = np.float64

__all__ = ["ModelClass", "ModelVibronic", "ModelVibronicPM", "ModelSampling", "BoxData",
           "BoxDataPM", "BoxResult", "BoxResultPM", "block_compute", "block_compute_pm"]

#: samples per fused launch; bounds the device memory of one call
LAUNCH_CHUNK = 1 << 22

SEP_KEYS = {"X": "number_of_samples", "nBlk": "number_of_blocks", "A": "number_of_states",
            "P": "number_of_beads", "N": "number_of_modes", "T": "temperature",
            "BlkS": "block_size", "dB": "delta_beta", "D": "id_data", "R": "id_rho",
            "beta": "beta", "tau": "tau"}   # server/server.py:11-23


def _torch():
    return _native.require_cuda()


def _dev(x, dtype=None):
    """numpy array / tensor -> contiguous CUDA FP64 (or dtype) tensor."""
    torch = _torch()
    dtype = dtype or torch.float64
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def _host(x):
    return x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)


# ---------------------------------------------------------------------------------------------
# model classes (pimc.py:59-424)
# ---------------------------------------------------------------------------------------------
class TemperatureDependentClass:
    """coth(tau w), csch(tau w) over (A,N) and the O-matrix prefactor exp(-tau Etilde_a) prod_j
    csch^(1/2) (pimc.py:59-89), on the device in FP64; ``omatrix`` is filled by build_o_matrix."""

    def __init__(self, model, tau):
        torch = _torch()
        A = model.states
        omega = np.broadcast_to(model.omega, (A, len(model.omega)))
        self.tau = tau
        self.cothAN = np.tanh(constants.hbar * tau * omega) ** (-1.0)
        self.cschAN = np.sinh(constants.hbar * tau * omega) ** (-1.0)
        energy = np.diag(model.energy) if model.energy.ndim > 1 else model.energy
        tilde = energy + model.delta_weight
        self.prefactor_A = np.exp(-tau * tilde) * np.prod(self.cschAN, axis=1) ** 0.5
        self.d_coth = torch.as_tensor(self.cothAN, dtype=torch.float64, device="cuda").contiguous()
        self.d_csch = torch.as_tensor(self.cschAN, dtype=torch.float64, device="cuda").contiguous()
        self.d_prefactor = torch.as_tensor(self.prefactor_A, dtype=torch.float64, device="cuda")
        self.omatrix = None
        self.omatrix_scaling = None


class ModelClass:
    """Model parameters (pimc.py:92-149)."""

    def __init__(self, states=1, modes=1):
        self.states, self.modes = states, modes
        self.omega = self.energy = self.linear = self.quadratic = None


class ModelVibronic(ModelClass):
    """Coupled model with the diagonal linear terms and energies folded into the oscillators
    (pimc.py:152-235)."""

    def __init__(self, data):
        super().__init__(data.states, data.modes)
        self.beta, self.tau = data.beta, data.tau

    def load_model(self, path):
        kw = vIO.load_model_from_JSON(path)
        self.states, self.modes = kw[VMK.A], kw[VMK.N]
        self.energy, self.omega = kw[VMK.E].copy(), kw[VMK.w].copy()
        self.linear, self.quadratic = kw[VMK.G1].copy(), kw[VMK.G2].copy()
        self.raw = kw

    def precompute(self, data):
        A = self.states
        self.delta_weight = np.array([-0.5 * (self.linear[:, a, a] ** 2 / self.omega).sum()
                                      for a in range(A)])              # pimc.py:172-177
        self.const = TemperatureDependentClass(self, self.tau)       # pimc.py:203-206
        self.state_shift = np.array([-self.linear[:, a, a] / self.omega for a in range(A)])
        for a in range(A):                                            # pimc.py:208-218
            self.linear[:, a, a] = 0.0
            self.energy[a, a] = 0.0


class ModelVibronicPM(ModelVibronic):
    """Plus/minus version: constants at beta +- delta_beta too (pimc.py:238-269)."""

    def __init__(self, data):
        super().__init__(data)
        self.delta_beta = data.delta_beta

    def precompute(self, data):
        self.beta_plus = self.beta + self.delta_beta
        self.beta_minus = self.beta - self.delta_beta
        self.tau_plus = self.beta_plus / data.beads
        self.tau_minus = self.beta_minus / data.beads
        A = self.states
        self.delta_weight = np.array([-0.5 * (self.linear[:, a, a] ** 2 / self.omega).sum()
                                      for a in range(A)])
        self.const = TemperatureDependentClass(self, self.tau)
        self.const_plus = TemperatureDependentClass(self, self.tau_plus)
        self.const_minus = TemperatureDependentClass(self, self.tau_minus)
        self.state_shift = np.array([-self.linear[:, a, a] / self.omega for a in range(A)])
        for a in range(A):
            self.linear[:, a, a] = 0.0
            self.energy[a, a] = 0.0


class ModelSampling(ModelClass):
    """Diagonal sampling model rho (pimc.py:272-424)."""

    def __init__(self, data):
        super().__init__(data.states, data.modes)
        self.beta, self.tau = data.beta, data.tau

    def load_model(self, path):
        kw = vIO.load_diagonal_model_from_JSON(path)
        self.states, self.modes = kw[VMK.A], kw[VMK.N]
        self.energy, self.omega = kw[VMK.E].copy(), kw[VMK.w].copy()
        self.linear, self.quadratic = kw[VMK.G1].copy(), kw[VMK.G2].copy()
        self.raw = kw

    def precompute(self, data):
        self.delta_weight = -0.5 * (self.linear ** 2 / self.omega[:, None]).sum(axis=0)
        w = np.exp(-self.beta * (self.energy + self.delta_weight))
        w /= np.prod(np.sinh(self.beta * self.omega / 2.0))
        self.state_weight = w / w.sum()                              # pimc.py:341-351
        self.const = TemperatureDependentClass(self, self.tau)
        self.state_shift = (-self.linear / self.omega[:, None]).T.copy()
        self.linear[:] = 0.0
        self.energy[:] = np.nan
        lam = data.circulant_eigvals
        self.inverse_covariance = (2.0 * self.const.cothAN[:, :, None]
                                   - self.const.cschAN[:, :, None] * lam[None, None, :])


# ---------------------------------------------------------------------------------------------
# BoxData (pimc.py:427-738)
# ---------------------------------------------------------------------------------------------
class BoxData:
    """Execution parameters, model constants and device plan of one run."""
    block_size = samples = blocks = 0
    states = modes = beads = 0
    temperature = beta = tau = 0.0
    delta_beta = None
    id_data = id_rho = 0
    path_vib_model = path_rho_model = ""
    hash_vib = hash_rho = None
    seed = None
    vib = rho = None
    _COMMA_REPLACEMENT = ";"
    _SEPARATORS = (_COMMA_REPLACEMENT, ":")

    def __init__(self):
        self._plan = None
        self._plan64 = None

    # ---- constructors (pimc.py:471-510) ----
    @classmethod
    def from_FileStructure(cls, FS):
        data = cls()
        data.id_data, data.id_rho = FS.id_data, FS.id_rho
        data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
        data.states, data.modes = vIO.extract_dimensions_of_model(FS)
        return data

    @classmethod
    def build(cls, id_data, id_rho):
        data = cls()
        data.id_data, data.id_rho = id_data, id_rho
        return data

    @classmethod
    def from_json_file(cls, path):
        with open(path, mode="r", encoding="UTF8") as fh:
            return cls.from_json_string(fh.read())

    @classmethod
    def from_json_string(cls, json_str):
        data = cls()
        data.load_json_string(json_str)
        return data

    @classmethod
    def json_serialize(cls, params):
        return json.dumps(params, separators=cls._SEPARATORS)

    def encode_self(self, params=None):
        """JSON parameters with ';' for ',' so the string survives SLURM env passing
        (pimc.py:517-540)."""
        if params is None:
            params = {SEP_KEYS["X"]: self.samples, SEP_KEYS["nBlk"]: self.blocks,
                      SEP_KEYS["A"]: self.states, SEP_KEYS["P"]: self.beads,
                      SEP_KEYS["N"]: self.modes, SEP_KEYS["T"]: self.temperature,
                      SEP_KEYS["BlkS"]: self.block_size, SEP_KEYS["dB"]: self.delta_beta,
                      SEP_KEYS["D"]: self.id_data, SEP_KEYS["R"]: self.id_rho,
                      SEP_KEYS["beta"]: self.beta, SEP_KEYS["tau"]: self.tau}
        return self.json_serialize(params)

    def load_json_string(self, json_str):
        """pimc.py:543-593."""
        params = json.loads(json_str.replace(self._COMMA_REPLACEMENT, ","))
        k = SEP_KEYS
        self.samples, self.blocks = params[k["X"]], params[k["nBlk"]]
        self.states, self.beads, self.modes = params[k["A"]], params[k["P"]], params[k["N"]]
        self.temperature, self.block_size = params[k["T"]], params[k["BlkS"]]
        self.id_data, self.id_rho = params[k["D"]], params[k["R"]]
        self.beta = params.get(k["beta"], 1.0 / (constants.boltzman * self.temperature))
        self.tau = params.get(k["tau"], self.beta / self.beads)
        if isinstance(params.get(k["dB"]), float):
            self.delta_beta = params[k["dB"]]
        FS = file_structure.FileStructure(params["path_root"], self.id_data, self.id_rho)
        self.path_vib_model, self.path_rho_model = FS.path_vib_model, FS.path_rho_model
        FS.generate_model_hashes()
        self.hash_vib, self.hash_rho = FS.hash_vib, FS.hash_rho

    # ---- preprocess (pimc.py:633-692) ----
    def _plus_minus(self):
        return False

    def initialize_models(self):
        vib_cls = ModelVibronicPM if self._plus_minus() else ModelVibronic
        self.vib = vib_cls(self)
        self.vib.load_model(self.path_vib_model)
        self.vib.precompute(self)
        self.rho = ModelSampling(self)
        self.rho.load_model(self.path_rho_model)
        self.rho.precompute(self)
        self.prepared = PreparedModels(self.vib.raw, self.rho.raw, self.beads, beta=self.beta,
                                       delta_beta=self.delta_beta if self._plus_minus() else None)
        self._plan = None
        self._plan64 = None

    def preprocess(self):
        A, N, P, B, X = self.states, self.modes, self.beads, self.block_size, self.samples
        self.param_dict = {"X": X, "A": A, "N": N, "P": P, "B": B}
        self.size_list = ["X", "P", "N", "A", "B", "XP", "BP", "AN", "NA", "AA", "BNP", "BPA",
                          "BAA", "XNP", "NAA", "NNA", "ANP", "BANP", "BPAA", "NNAA", "BPAN"]
        self.size = {key: tuple(self.param_dict[c] for c in key) for key in self.size_list}
        self.beta = constants.beta(self.temperature)
        self.tau = self.beta / self.beads
        assert self.beads >= 3, "circulant matrix requires 3 or more beads"
        first = np.zeros(P)
        first[1] = first[-1] = 1.0
        idx = (np.arange(P)[:, None] - np.arange(P)[None, :]) % P
        self.circulant_matrix = first[idx]
        self.circulant_eigvals, self.circulant_eigvects = np.linalg.eigh(self.circulant_matrix, UPLO="L")
        if self.seed is None:
            self.seed = int(np.random.randint(0, 2 ** 62, dtype=np.int64))
        self.initialize_models()
        self.qTensor = None
        self.qTempTensor = None

    # ---- device plans ----
    @property
    def plan(self):
        if self._plan is None:
            self._plan = DevicePlan(self.prepared, precision=32)
        return self._plan

    @property
    def plan64(self):
        if self._plan64 is None:
            self._plan64 = DevicePlan(self.prepared, precision=64)
        return self._plan64

    # ---- sampling (pimc.py:595-631) ----
    def draw_sample(self, sample_view):
        """Draw the block's bead coordinates on the device (Philox stream of data.seed, sample
        counter = global sample index); the reference's draw_sample + the normal-mode part of
        transform_sampled_coordinates (pimc.py:326-334, 618-621)."""
        torch = _torch()
        start, stop = sample_view.start or 0, sample_view.stop
        n = stop - start
        q = torch.empty((n, self.modes, self.beads), dtype=torch.float32, device="cuda")
        src = torch.empty((n,), dtype=torch.int32, device="cuda")
        lib = _native.load()
        _native.check(lib.pbr_sample_q(self.plan.struct, self.seed, start, n, _native.ptr(q),
                                       _native.ptr(src), _native.stream_handle()), "draw_sample")
        self._block_q, self._block_src = q, src

    def transform_sampled_coordinates(self, sample_view):
        """Broadcast the block's q over the surface slots (pimc.py:613-631)."""
        q = self._block_q.to(dtype=_torch().float64)
        self.qTensor = q[:, None, :, :].expand(-1, self.states, -1, -1).contiguous()
        self.qTempTensor = q[:, None, :, :].expand(-1, self.rho.states, -1, -1).contiguous()

    def generate_random_R_values(self, result, storage_array, sample_view):
        """Uniform [0,1) R (pimc.py:602-611): slots hold q = R - d_a."""
        R = np.random.random(size=(sample_view.stop - sample_view.start, self.modes, self.beads))
        storage_array[sample_view] = R
        self.qTensor = _dev(R[:, None, :, :] - self.vib.state_shift[None, :, :, None])


class BoxDataPM(BoxData):
    """Plus/minus version (pimc.py:695-738)."""

    def __init__(self, delta_beta=None):
        super().__init__()
        self.delta_beta = constants.delta_beta if delta_beta is None else delta_beta

    def _plus_minus(self):
        return True

    def preprocess(self):
        self.beta = constants.beta(self.temperature)
        self.beta_plus = self.beta + self.delta_beta
        self.beta_minus = self.beta - self.delta_beta
        self.tau_plus = self.beta_plus / self.beads
        self.tau_minus = self.beta_minus / self.beads
        super().preprocess()


# ---------------------------------------------------------------------------------------------
# results (pimc.py:741-1040)
# ---------------------------------------------------------------------------------------------
class BoxResult:
    """Per-sample FP64 results, NaN-initialised, and their ``.npz`` file."""
    id_job = None
    hash_vib = hash_rho = None
    key_list = ["number_of_samples", "s_rho", "s_g"]

    def __init__(self, data=None, X=None):
        if data is not None:
            self.partial_name = partial(file_structure.pimc().format, P=data.beads, T=data.temperature)
            self.samples = data.samples
            self.hash_vib, self.hash_rho = data.hash_vib, data.hash_rho
        elif X is not None:
            self.samples = X
        else:
            self.samples = 0
        self.device = {}
        self.initialize_arrays()

    def initialize_arrays(self):
        self.scaled_g = np.full(self.samples, np.nan, dtype=F64)
        self.scaled_rho = np.full(self.samples, np.nan, dtype=F64)

    @classmethod
    def read_number_of_samples(cls, path_full):
        with np.load(path_full, mmap_mode="r") as d:
            return d["number_of_samples"]

    @classmethod
    def verify_result_keys_are_present(cls, path, fileObj):
        for k in cls.key_list:
            if k not in fileObj.keys():
                raise AssertionError(f"Expected key ({k}) not present in result file\n{path}\n")

    @classmethod
    def result_keys_are_present_in(cls, iterable):
        return all(k in iterable for k in cls.key_list)

    def compute_path_to_file(self):
        if self.samples == 0:
            raise AssertionError(f"{self.__class__.__name__} still has 0 samples - this should not happen")
        J = int(self.id_job) if self.id_job is not None else 0
        self.name = self.partial_name(J=J)
        return os.path.join(self.path_root, self.name)

    def _payload(self):
        return {"hash_vib": self.hash_vib, "hash_rho": self.hash_rho,
                "number_of_samples": self.samples, "s_rho": self.scaled_rho, "s_g": self.scaled_g}

    def save_results(self, number_of_samples):
        path = self.compute_path_to_file()
        assert self.hash_vib is not None and self.hash_rho is not None, \
            "we save hash values if they don't exist!"
        np.savez(path, **self._payload())

    def load_results(self, path):
        with np.load(path, mmap_mode="r") as d:
            self.verify_result_keys_are_present(path, d)
            if self.samples == 0:
                self.samples = int(d["number_of_samples"])
            elif int(d["number_of_samples"]) != self.samples:
                raise AssertionError("BoxResult has a different number of samples that the input file - this should not happen")
            self.initialize_arrays()
            self._fill(d, 0, self.samples)

    def _fill(self, d, start, length):
        self.scaled_g[start:start + length] = d["s_g"][:length]
        self.scaled_rho[start:start + length] = d["s_rho"][:length]

    def load_multiple_results(self, list_of_paths, desired_number_of_samples=None):
        """Merge result files (pimc.py:853-912 / 975-1040): files missing a key are skipped,
        samples are additive across files, zeros in rho are rejected."""
        assert len(list_of_paths) != 0, "list_of_paths cannot be empty"
        total, good = 0, []
        try:
            for path in list_of_paths:
                with np.load(path, mmap_mode="r") as d:
                    if self.result_keys_are_present_in(d.keys()):
                        total += int(d["number_of_samples"])
                        good.append(path)
        except Exception as err:
            print("Did we get another mangled .npz file?")
            raise err
        assert len(good) > 0, f"none of the provided paths were good, i.e. none of them had all the required keys {self.key_list}"
        assert total != 0, "number of samples should have changed"
        if desired_number_of_samples is None:
            desired_number_of_samples = total
        elif total >= desired_number_of_samples:
            total = desired_number_of_samples
        else:
            print("We found less samples than were requested!!")
        self.samples = total
        self.initialize_arrays()
        start = 0
        for path in sorted(good):
            if start >= desired_number_of_samples:
                break
            with np.load(path) as d:
                length = min(int(d["number_of_samples"]), desired_number_of_samples - start)
                assert not np.any(d["s_rho"][0:length] == 0.0), "Zeros in the denominator"
                self._fill(d, start, length)
                start += length


class BoxResultPM(BoxResult):
    key_list = ["s_gP", "s_gM"] + BoxResult.key_list

    def initialize_arrays(self):
        super().initialize_arrays()
        self.scaled_gofr_plus = np.full(self.samples, np.nan, dtype=F64)
        self.scaled_gofr_minus = np.full(self.samples, np.nan, dtype=F64)

    def _payload(self):
        d = super()._payload()
        d.update(s_gP=self.scaled_gofr_plus, s_gM=self.scaled_gofr_minus)
        return d

    def _fill(self, d, start, length):
        super()._fill(d, start, length)
        self.scaled_gofr_plus[start:start + length] = d["s_gP"][:length]
        self.scaled_gofr_minus[start:start + length] = d["s_gM"][:length]


# ---------------------------------------------------------------------------------------------
# fused block evaluation
# ---------------------------------------------------------------------------------------------
def evaluate_device(plan, X, seed=None, offset=0, q=None, plus_minus=True, want_q=False,
                    want_coef=False, stream=None):
    """Run the fused kernel on X samples; returns a dict of CUDA tensors s_rho, s_g (, s_gp, s_gm,
    g_coef, log_scale, q, src).  With ``q`` (CUDA tensor [X,N,P], FP64 or FP32) the caller's bead
    coordinates are evaluated instead of drawing samples."""
    torch = _torch()
    lib = _native.load()
    prep = plan.prep
    K = prep.K
    dev = torch.device("cuda")
    out = {k: torch.empty(X, dtype=torch.float64, device=dev) for k in ("s_rho", "s_g", "log_scale")}
    if K > 0:
        out["s_gp"] = torch.empty(X, dtype=torch.float64, device=dev)
        out["s_gm"] = torch.empty(X, dtype=torch.float64, device=dev)
    if want_coef:
        out["g_coef"] = torch.empty((X, K + 1), dtype=torch.float64, device=dev)
    if want_q and q is None:
        out["q"] = torch.empty((X, prep.N, prep.P), dtype=torch.float32, device=dev)
        out["src"] = torch.empty(X, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    o = _native.PbrOutputs()
    for name, key in (("s_rho", "s_rho"), ("s_g", "s_g"), ("s_gp", "s_gp"), ("s_gm", "s_gm"),
                      ("g_coef", "g_coef"), ("log_scale", "log_scale"), ("q_out", "q"),
                      ("src_out", "src")):
        setattr(o, name, out[key].data_ptr() if key in out else None)
    o.status = status.data_ptr()
    sh = _native.stream_handle(stream)
    def launch(use_tc):
        qq = q.float() if (use_tc and q is not None and q.dtype == torch.float64) else q
        if qq is None and use_tc:
            scratch = plan.tc_scratch()
            return lib.pbr_sample_eval_tc(plan.struct, int(seed), int(offset), int(X), o, scratch.data_ptr(),
                                          scratch.numel(), sh)
        if qq is None:
            return lib.pbr_sample_eval(plan.struct, int(seed), int(offset), int(X), o, sh)
        if qq.dtype == torch.float64:
            return lib.pbr_eval_q(plan.struct, _native.ptr(qq), int(X), o, sh)
        if use_tc:
            scratch = plan.tc_scratch()
            return lib.pbr_eval_q_tc(plan.struct, _native.ptr(qq), int(X), o, scratch.data_ptr(), scratch.numel(), sh)
        return lib.pbr_eval_q_f32(plan.struct, _native.ptr(qq), int(X), o, sh)

    use_tc = getattr(plan, "use_tc", False)
    rc = launch(use_tc)
    if (rc == _native.PBR_ERR_UNSUPPORTED and not use_tc and plan.precision == 32
            and plan.variant == plan.VARIANT_AUTO):
        # a shape the shared-memory forms cannot hold: the tensor-core form from now on
        plan.use_tc = True
        rc = launch(True)
    _native.check(rc, "fused block evaluation")
    out["status"] = status
    return out


def _run_blocks(data, result, plus_minus):
    torch = _torch()
    X = data.blocks * data.block_size
    plan = data.plan
    dev = {k: [] for k in ("s_rho", "s_g", "s_gp", "s_gm")}
    for start in range(0, X, LAUNCH_CHUNK):
        n = min(LAUNCH_CHUNK, X - start)
        out = evaluate_device(plan, n, seed=data.seed, offset=start, plus_minus=plus_minus)
        if int(out["status"].item()) != 0:
            raise AssertionError("non-finite g or rho in the fused evaluation")
        for k in dev:
            if k in out:
                dev[k].append(out[k])
    cat = {k: torch.cat(v) for k, v in dev.items() if v}
    result.device = cat
    result.scaled_rho[:X] = _host(cat["s_rho"])
    result.scaled_g[:X] = _host(cat["s_g"])
    if plus_minus:
        result.scaled_gofr_plus[:X] = _host(cat["s_gp"])
        result.scaled_gofr_minus[:X] = _host(cat["s_gm"])
    return X


def block_compute(data, result):
    """rho and g for all samples, scaled by prod_p 1/S12 (pimc.py:1341-1385)."""
    end = _run_blocks(data, result, plus_minus=False)
    result.save_results(end)


def block_compute_pm(data, result):
    """rho, g, g(beta+db), g(beta-db) for all samples (pimc.py:1388-1462)."""
    assert isinstance(data, BoxDataPM), "incorrect object type"
    assert isinstance(result, BoxResultPM), "incorrect object type"
    end = _run_blocks(data, result, plus_minus=True)
    result.save_results(end)


# ---------------------------------------------------------------------------------------------
# stage functions on device tensors (pimc.py:1062-1213)
# ---------------------------------------------------------------------------------------------
def _slots_for(data, state_shift):
    q = data.qTensor if state_shift.shape[0] == data.qTensor.shape[1] else data.qTempTensor
    return _dev(q)


def build_o_matrix(data, model, state_shift):
    """model.omatrix[B,P,Am,Am] (pimc.py:1087-1129)."""
    torch = _torch()
    lib = _native.load()
    q = _slots_for(data, state_shift)
    B, Am, N, P = q.shape
    shift = _dev(state_shift)
    O = torch.empty((B, P, Am, Am), dtype=torch.float64, device="cuda")
    n_fill = min(data.states, Am)
    _native.check(lib.pbr_o_matrix(_native.ptr(q), B, Am, N, P, _native.ptr(model.d_coth),
                                   _native.ptr(model.d_csch), _native.ptr(shift),
                                   _native.ptr(model.d_prefactor), n_fill, _native.ptr(O),
                                   _native.stream_handle()), "build_o_matrix")
    model.omatrix = O


def build_scaling_factors(S12, model_one, model_two):
    """Each model's max O entry per (sample, bead) and S12, the larger of the two
    (pimc.py:1076-1084), by the library's pbr_scaling_factors."""
    torch = _torch()
    lib = _native.load()
    O1, O2 = model_one.omatrix, model_two.omatrix
    B, P, A1, _ = O1.shape
    A2 = O2.shape[2]
    assert O2.shape[:2] == (B, P), "both models' O matrices must cover the same samples and beads"
    model_one.omatrix_scaling = torch.empty((B, P), dtype=torch.float64, device="cuda")
    model_two.omatrix_scaling = torch.empty((B, P), dtype=torch.float64, device="cuda")
    s = torch.empty((B, P), dtype=torch.float64, device="cuda")
    _native.check(lib.pbr_scaling_factors(_native.ptr(O1), A1, _native.ptr(O2), A2, B, P,
                                          _native.ptr(model_one.omatrix_scaling),
                                          _native.ptr(model_two.omatrix_scaling), _native.ptr(s),
                                          _native.stream_handle()), "build_scaling_factors")
    if hasattr(S12, "copy_"):
        S12.copy_(s)
    else:
        S12[...] = _host(s)
    return s


def scale_o_matrices(scalingFactor, model_one, model_two):
    """Divide both models' O by S12 (pimc.py:1062-1066)."""
    lib = _native.load()
    s = _dev(scalingFactor)
    for m in (model_one, model_two):
        B, P, A, _ = m.omatrix.shape
        _native.check(lib.pbr_divide_o_matrix(_native.ptr(m.omatrix), A, B, P, _native.ptr(s),
                                              _native.stream_handle()), "scale_o_matrices")


def _store(outputArray, idx, values):
    if hasattr(outputArray, "copy_"):
        outputArray[idx] = values
    else:
        outputArray[idx] = _host(values)


def build_denominator(rho_model, outputArray, idx):
    """rho = Tr prod_p O^rho (pimc.py:1132-1136)."""
    torch = _torch()
    lib = _native.load()
    O = rho_model.omatrix
    B, P, A, _ = O.shape
    out = torch.empty(B, dtype=torch.float64, device="cuda")
    _native.check(lib.pbr_denominator(_native.ptr(O), B, A, P, _native.ptr(out),
                                      _native.stream_handle()), "build_denominator")
    _store(outputArray, idx, out)


def diagonalize_coupling_matrix(data):
    """V(q) and its eigen-decomposition (pimc.py:1139-1174)."""
    torch = _torch()
    lib = _native.load()
    q = _dev(data.qTensor)
    B, A, N, P = q.shape
    vib = data.vib
    E, L, Q = _dev(vib.energy), _dev(vib.linear), _dev(vib.quadratic)
    data.coupling_matrix = torch.empty((B, P, A, A), dtype=torch.float64, device="cuda")
    data.coupling_eigvals = torch.empty((B, P, A), dtype=torch.float64, device="cuda")
    data.coupling_eigvects = torch.empty((B, P, A, A), dtype=torch.float64, device="cuda")
    ok = torch.ones(1, dtype=torch.int32, device="cuda")
    _native.check(lib.pbr_coupling_eigh(_native.ptr(q), B, A, N, P, _native.ptr(E), _native.ptr(L),
                                        _native.ptr(Q), _native.ptr(data.coupling_matrix),
                                        _native.ptr(data.coupling_eigvals),
                                        _native.ptr(data.coupling_eigvects), _native.ptr(ok),
                                        _native.stream_handle()), "diagonalize_coupling_matrix")
    assert int(ok.item()) == 1, "coupling matrix is not symmetric"


def build_numerator(data, vib, outputArray, idx):
    """M = U exp(-tau lambda) U^T with the central tau, g = Tr prod_p M_p O_p (pimc.py:1177-1213)."""
    torch = _torch()
    lib = _native.load()
    B, P, A = data.coupling_eigvals.shape
    data.M_matrix = torch.empty((B, P, A, A), dtype=torch.float64, device="cuda")
    out = torch.empty(B, dtype=torch.float64, device="cuda")
    _native.check(lib.pbr_numerator(_native.ptr(data.coupling_eigvals),
                                    _native.ptr(data.coupling_eigvects), _native.ptr(vib.omatrix),
                                    B, A, P, float(data.tau), _native.ptr(data.M_matrix),
                                    _native.ptr(out), _native.stream_handle()), "build_numerator")
    _store(outputArray, idx, out)


# ---------------------------------------------------------------------------------------------
# learned-proposal data path (pimc.py:1216-1338)
# ---------------------------------------------------------------------------------------------
def block_compute_gR(data, result):
    """Unscaled g on rho samples, per block (pimc.py:1216-1247)."""
    vib = data.vib
    end = 0
    for blk in range(data.blocks):
        view = slice(blk * data.block_size, (blk + 1) * data.block_size)
        data.draw_sample(view)
        data.transform_sampled_coordinates(view)
        build_o_matrix(data, vib.const, vib.state_shift)
        diagonalize_coupling_matrix(data)
        build_numerator(data, vib.const, result.scaled_g, view)
        end = view.stop
    result.save_results(end)


def save_gR_with_samples(data, result, input_R_values):
    """Training files P{P}_T{T}_J{J}_training_data_{g_output,input}.npz (pimc.py:1250-1270)."""
    result.partial_name = partial(file_structure.training_data_g_output().format, P=data.beads,
                                  T=data.temperature)
    np.savez(result.compute_path_to_file(), number_of_samples=result.samples, g=result.scaled_g)
    result.partial_name = partial(file_structure.training_data_input().format, P=data.beads,
                                  T=data.temperature)
    np.savez(result.compute_path_to_file(), number_of_samples=result.samples,
             input_R_values=input_R_values)


def block_compute_rhoR_from_input_samples(data, result, input_R_values):
    """rho(R) on given R (pimc.py:1273-1302): slots R - d^vib_a, rho O matrix on them."""
    assert data.rho.states == data.states, \
        "rho(R) needs a sampling model with the vibronic surface count"
    rho = data.rho
    for blk in range(data.blocks):
        view = slice(blk * data.block_size, (blk + 1) * data.block_size)
        R = np.asarray(input_R_values[view])
        data.qTensor = _dev(R[:, None, :, :] - data.vib.state_shift[None, :, :, None])
        build_o_matrix(data, rho.const, rho.state_shift)
        build_denominator(rho.const, result.scaled_rho, view)


def block_compute_gR_from_raw_samples(data, result):
    """g(R) on uniform random R and the training files (pimc.py:1305-1338)."""
    vib = data.vib
    R_all = np.empty((data.samples, data.modes, data.beads), dtype=F64)
    for blk in range(data.blocks):
        view = slice(blk * data.block_size, (blk + 1) * data.block_size)
        data.generate_random_R_values(result, R_all, view)
        build_o_matrix(data, vib.const, vib.state_shift)
        diagonalize_coupling_matrix(data)
        build_numerator(data, vib.const, result.scaled_g, view)
    save_gR_with_samples(data, result, R_all)


def normal_mode_basis(P):
    """The ring normal-mode basis the device sampler uses (orthonormal, columns = modes)."""
    return ring_mode_basis(P)
