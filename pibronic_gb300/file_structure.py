"""Directory layout and file names of a data set (pibronic/data/file_structure.py:33-140,
pibronic/data/file_name.py:38-140): data_set_{D}/[rho_{R}/]{parameters,results,...}/ with model
files coupled_model.json / sampling_model.json and result files P{P}_T{T:.2f}_J{J}_data_points.npz."""
from __future__ import annotations

import os
from os.path import join

from . import vibronic_io as vIO

coupled_model = "coupled_model.json"
harmonic_model = "harmonic_model.json"
sampling_model = "sampling_model.json"
analytic_results = "analytic_results.json"
original_model = "original_coupled_model.json"
iterative_model = "iterative_model.json"
iterative_matrix = "iterative_matrix.txt"
original_analytic_results = "original_analytic_results.json"
orthogonal_matrix = "orthogonal_matrix.npy"


def pimc(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    """Result file name of one job (file_name.py:38-46)."""
    return "P{:s}_T{:s}_J{:s}_data_points.npz".format(P, T, J)


def jackknife(P="{P:d}", T="{T:.2f}", X="{X:d}"):
    """Estimator output name (file_name.py:55-62)."""
    return "P{:s}_T{:s}_X{:s}_thermo".format(P, T, X)


def sos(B="{B:d}"):
    """Sum-over-states results of one basis size (file_name.py:68-78)."""
    return "sos_B{:s}.json".format(B)


def trotter(P="{P:d}", B="{B:d}"):
    """Trotter results of one bead count and basis size (file_name.py:82-95)."""
    return "trotter_P{:s}_B{:s}.json".format(P, B)


def training_data_input(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    return "P{:s}_T{:s}_J{:s}_training_data_input.npz".format(P, T, J)


def training_data_g_output(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    return "P{:s}_T{:s}_J{:s}_training_data_g_output.npz".format(P, T, J)


def training_data_rho_output(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    return "P{:s}_T{:s}_J{:s}_training_data_rho_output.npz".format(P, T, J)


class FileStructure:
    """Paths of one (data set, sampling model) pair; creates the directories unless told not to."""

    SUB_DIRS = ("parameters", "results", "execution_output", "plots")

    def __init__(self, path_root, id_data, id_rho=0, no_makedir=False):
        """file_structure.py:60-135; with no_makedir the object only holds the path strings."""
        assert os.path.exists(path_root), f"the path_root ({path_root}) does not exist"
        assert os.path.isdir(path_root), f"the path_root ({path_root}) is not a directory"
        self.id_data, self.id_rho = id_data, id_rho
        self.path_root = os.path.abspath(path_root)
        vib = join(self.path_root, f"data_set_{id_data:d}")
        self.path_data = vib + "/"
        self.path_es = join(vib, "electronic_structure")
        self.path_vib_params = join(vib, "parameters") + "/"
        self.path_vib_results = join(vib, "results") + "/"
        self.path_vib_output = join(vib, "execution_output") + "/"
        self.path_vib_plots = join(vib, "plots") + "/"
        self._set_rho_paths(id_rho)
        self.dir_list = ["path_data", "path_es", "path_vib_params", "path_vib_results", "path_vib_output",
                         "path_vib_plots", "path_rho", "path_rho_params", "path_rho_results",
                         "path_rho_output", "path_rho_plots"]
        self.template_sos_vib = self.path_vib_params + sos()
        self.template_trotter_vib = self.path_vib_params + trotter()
        self.path_vib_model = join(self.path_vib_params, coupled_model)
        self.path_har_model = join(self.path_vib_params, harmonic_model)
        self.path_iter_model = join(self.path_vib_params, iterative_model)
        self.path_iter_mat = join(self.path_vib_params, iterative_matrix)
        self.path_analytic_vib = join(self.path_vib_params, analytic_results)
        self.path_analytic_orig = join(self.path_vib_params, original_analytic_results)
        self.path_orig_model = join(self.path_vib_params, original_model)
        self.path_ortho_mat = join(self.path_vib_params, orthogonal_matrix)
        if not no_makedir:
            self.make_directories()

    def _set_rho_paths(self, id_rho):
        rho = join(self.path_root, f"data_set_{self.id_data:d}", f"rho_{id_rho:d}")
        self.path_rho = rho + "/"
        self.path_rho_params = join(rho, "parameters") + "/"
        self.path_rho_results = join(rho, "results") + "/"
        self.path_rho_output = join(rho, "execution_output") + "/"
        self.path_rho_plots = join(rho, "plots") + "/"
        self.template_pimc = self.path_rho_results + pimc(J="{J:s}")
        self.template_jackknife = self.path_rho_results + jackknife()
        self.template_sos_rho = self.path_rho_params + sos()
        self.path_rho_model = join(self.path_rho_params, sampling_model)
        self.path_analytic_rho = join(self.path_rho_params, analytic_results)

    def make_rho_directories(self, id_rho):
        """The sub-directories of another sampling model of this data set (file_structure.py:160-176)."""
        if id_rho == self.id_rho:
            self.make_directories()
            return
        rho = join(self.path_root, f"data_set_{self.id_data:d}", f"rho_{id_rho:d}")
        for sub in self.SUB_DIRS:
            os.makedirs(join(rho, sub), exist_ok=True)

    def change_rho(self, id_rho):
        """Point the sampling-model paths at another rho of the data set, creating its directories
        (file_structure.py:178-207).  As in the reference, id_rho and path_rho are left as they were."""
        self.make_rho_directories(id_rho)
        path_rho = self.path_rho
        self._set_rho_paths(id_rho)
        self.path_rho = path_rho

    @classmethod
    def from_boxdata(cls, path_root, data):
        return cls(path_root, data.id_data, data.id_rho)

    def make_directories(self):
        for attr in self.dir_list:
            os.makedirs(getattr(self, attr), exist_ok=True)

    def directories_exist(self):
        return all(os.path.isdir(getattr(self, a)) for a in self.dir_list)

    def generate_model_hashes(self, force_flag=False):
        if hasattr(self, "hash_vib") and hasattr(self, "hash_rho") and not force_flag:
            return
        self.hash_vib = vIO.create_model_hash(FS=self)
        self.hash_rho = vIO.create_diagonal_model_hash(FS=self)
