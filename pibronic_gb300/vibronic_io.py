"""Model files: the reference's JSON format for coupled (vibronic) and diagonal (sampling) models.

Format (pibronic/vibronic/vibronic_model_io.py:42-73, 517-626; keys
vibronic_model_keys.py:9-26): a JSON object with "number of modes" N, "number of surfaces" A,
"energies" E, "frequencies" w, "linear couplings" G1, "quadratic couplings" G2.  Coupled shapes:
E (A,A), w (N,), G1 (N,A,A), G2 (N,N,A,A); diagonal shapes: E (A,), G1 (N,A), G2 (N,N,A).  A
coupling array that is all zero is omitted on save and read back as zeros.
"""
from __future__ import annotations

import copy
import enum
import hashlib
import json
import os
import shutil

import numpy as np

F64 = np.float64


class VibronicModelKeys(enum.Enum):
    """JSON keys of the model files (vibronic_model_keys.py:6-26)."""
    number_of_modes = "number of modes"
    number_of_surfaces = "number of surfaces"
    energies = "energies"
    frequencies = "frequencies"
    linear_couplings = "linear couplings"
    quadratic_couplings = "quadratic couplings"
    cubic_couplings = "cubic couplings"
    quartic_couplings = "quartic couplings"
    N = "number of modes"
    A = "number of surfaces"
    E = "energies"
    w = "frequencies"
    G1 = "linear couplings"
    G2 = "quadratic couplings"
    G3 = "cubic couplings"
    G4 = "quartic couplings"


VMK = VibronicModelKeys


def model_shape_dict(A, N):
    """Array shapes of a coupled model (vibronic_model_io.py:42-56)."""
    return {VMK.E: (A, A), VMK.w: (N,), VMK.G1: (N, A, A), VMK.G2: (N, N, A, A),
            VMK.G3: (N, N, N, A, A), VMK.G4: (N, N, N, N, A, A)}


def diagonal_model_shape_dict(A, N):
    """Array shapes of a diagonal model (vibronic_model_io.py:59-73)."""
    return {VMK.E: (A,), VMK.w: (N,), VMK.G1: (N, A), VMK.G2: (N, N, A),
            VMK.G3: (N, N, N, A), VMK.G4: (N, N, N, N, A)}


def _read(path):
    with open(path, mode="r", encoding="UTF8") as fh:
        return _parse(fh.read())


def _parse(text):
    return {VMK(k): v for k, v in json.loads(text).items()}


def _dims(d):
    return int(d[VMK.A]), int(d[VMK.N])


def _load(path, shapes_of, text=None):
    raw = _parse(text) if text is not None else _read(path)
    A, N = _dims(raw)
    shapes = shapes_of(A, N)
    out = {VMK.N: N, VMK.A: A}
    for key in (VMK.E, VMK.w, VMK.G1, VMK.G2):
        arr = np.zeros(shapes[key], dtype=F64)
        if key in raw:
            arr[...] = np.array(raw[key], dtype=F64)
        out[key] = arr
    for key in (VMK.G3, VMK.G4):
        if key in raw:
            out[key] = np.array(raw[key], dtype=F64).reshape(shapes[key])
    return out


def load_model_from_JSON(path):
    """Coupled model dict with every array present (missing ones zero); vibronic_model_io.py:599."""
    model = _load(path, model_shape_dict)
    verify_model_parameters(model)
    return model


def load_diagonal_model_from_JSON(path):
    """Diagonal model dict (vibronic_model_io.py:626)."""
    model = _load(path, diagonal_model_shape_dict)
    verify_diagonal_model_parameters(model)
    return model


def _verify(d, shapes_of):
    assert VMK.N in d, "need the number of modes"
    assert VMK.A in d, "need the number of surfaces"
    shapes = shapes_of(*_dims(d))
    for key, value in d.items():
        if key in shapes and isinstance(value, np.ndarray):
            assert value.shape == shapes[key], f"{key} have incorrect shape"


def model_from_text(text, diagonal=False):
    """A model dict from JSON text (same rules as the file loaders)."""
    if diagonal:
        model = _load(None, diagonal_model_shape_dict, text=text)
        verify_diagonal_model_parameters(model)
    else:
        model = _load(None, model_shape_dict, text=text)
        verify_model_parameters(model)
    return model


def verify_model_parameters(d):
    _verify(d, model_shape_dict)


def verify_diagonal_model_parameters(d):
    _verify(d, diagonal_model_shape_dict)


def _save(path, d):
    out = {}
    for key, value in copy.deepcopy(d).items():
        name = key.value if isinstance(key, VMK) else key
        if isinstance(value, (np.ndarray, np.generic)):
            if np.count_nonzero(value) > 0:
                out[name] = np.asarray(value).tolist()
        else:
            out[name] = value
    with open(path, mode="w", encoding="UTF8") as fh:
        fh.write(json.dumps(out))


def save_model_to_JSON(path, d):
    verify_model_parameters(d)
    _save(path, d)


def save_diagonal_model_to_JSON(path, d):
    verify_diagonal_model_parameters(d)
    _save(path, d)


def extract_dimensions_of_model(FS=None, path=None):
    """(A, N) of a coupled model file."""
    path = FS.path_vib_model if FS is not None else path
    return _dims(_read(path))


def extract_dimensions_of_diagonal_model(FS=None, path=None):
    path = FS.path_rho_model if FS is not None else path
    return _dims(_read(path))


def _hash(string):
    """SHA-512 hex digest of a string's UTF-8 bytes (vibronic_model_io.py:293-297)."""
    return hashlib.sha512(string.encode("UTF-8")).hexdigest()


def _hash_file(path):
    assert os.path.isfile(path), f"The path provided is not a valid file! Path:\n{path}"
    with open(path, mode="r", encoding="UTF8") as fh:
        return _hash(fh.read())


def create_model_hash(FS=None, path=None):
    """SHA-512 of the coupled model file text (vibronic_model_io.py:293-311)."""
    return _hash_file(FS.path_vib_model if FS is not None else path)


def create_diagonal_model_hash(FS=None, path=None):
    """SHA-512 of the sampling model file text (vibronic_model_io.py:314-331)."""
    return _hash_file(FS.path_rho_model if FS is not None else path)


def remove_coupling_from_model(path_source, path_destination):
    """Diagonal model from the surface diagonal of a coupled one (vibronic_model_io.py:749-761)."""
    model = load_model_from_JSON(path_source)
    for key, value in list(model.items()):
        if isinstance(value, np.ndarray) and value.ndim >= 2:
            model[key] = np.diagonal(value, axis1=value.ndim - 2, axis2=value.ndim - 1).copy()
    save_diagonal_model_to_JSON(path_destination, model)


def create_harmonic_model(FS):
    """The coupled model without its off-diagonal couplings (vibronic_model_io.py:764-771)."""
    remove_coupling_from_model(FS.path_vib_model, FS.path_har_model)
    return FS.path_har_model


def create_basic_diagonal_model(FS):
    """The simplest sampling model: the harmonic (diagonal) part of the coupled model
    (vibronic_model_io.py:774-787)."""
    shutil.copyfile(create_harmonic_model(FS), FS.path_rho_model)
    return FS.path_rho_model
