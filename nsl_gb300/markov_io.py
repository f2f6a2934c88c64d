"""Markov-chain files without HDF5: the node layout of NSL's H5IO (src/NSL/IO/h5_io.tpp:68-307) as a directory tree.

NSL writes every saved Markov state of an HMC run to an HDF5 file through HighFive:

    <baseNode>/<n>/<field>                     the configuration's fields (e.g. phi), flattened, with the attributes
                                               "shape" and "type" (h5_io.tpp:243-307)
    <baseNode>/<n>/actVal                      the action value (complex for complex Type)
    <baseNode>/<n>/acceptanceProbability       double
    <baseNode>/<n>/acceptanceRate              the accepted flag as an integer
    <baseNode>/<n>/weights/<key>               additional weights
    <baseNode>/<n>/markovTime                  int

(h5_io.tpp:68-167), and HMC::generate resumes a chain from the highest-numbered state, dropping a state it cannot
read and going back one (HMC.tpp:57-110). HDF5 and HighFive are not available to this library, so MarkovChainFile
keeps the same node names as a directory tree under `root`, one `.npy` file per dataset (array, dtype and shape in
the file; a tensor dataset also keeps its shape and element type in a small `.attrs.json` beside it, as the HDF5
attributes). A dataset is written to a temporary file and renamed, so a state is either readable or detectably
incomplete. Node paths map one to one onto HDF5 dataset paths for a converter wherever h5py is installed.
"""
from __future__ import annotations

import json
import os
import shutil

import numpy as np

from .configuration import Configuration


class MarkovChainFile:
    """H5IO's interface for Markov states (exist, getMinMaxConfigs, write, read, deleteData) on a directory tree."""

    def __init__(self, root: str):
        self.root = os.path.abspath(root)
        os.makedirs(self.root, exist_ok=True)

    # ---- nodes ------------------------------------------------------------------------------------------------------
    def _path(self, node: str) -> str:
        parts = [p for p in node.strip("/").split("/") if p]
        if any(p in (".", "..") for p in parts):
            raise ValueError(f"invalid node {node!r}")
        return os.path.join(self.root, *parts)

    def exist(self, node: str) -> bool:
        """H5IO::exist: a group or a dataset of that name."""
        p = self._path(node)
        return os.path.isdir(p) or os.path.isfile(p + ".npy")

    def deleteData(self, node: str) -> None:
        """H5IO::deleteData: removes a group (with everything below it) or a dataset."""
        p = self._path(node)
        if os.path.isdir(p):
            shutil.rmtree(p)
        for ext in (".npy", ".attrs.json"):
            if os.path.isfile(p + ext):
                os.remove(p + ext)

    def getMinMaxConfigs(self, node: str) -> tuple[int, int]:
        """h5_io.tpp:44-66: the smallest and largest configuration number stored under node."""
        ids = [int(n) for n in os.listdir(self._path(node)) if n.isdigit() and os.path.isdir(self._path(f"{node}/{n}"))]
        if not ids:
            raise FileNotFoundError(f"no configurations under {node!r}")
        return min(ids), max(ids)

    # ---- datasets ---------------------------------------------------------------------------------------------------
    def _write_array(self, node: str, value, attrs: dict | None = None) -> None:
        p = self._path(node)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp.npy"
        np.save(tmp, np.asarray(value), allow_pickle=False)
        os.replace(tmp, p + ".npy")
        if attrs is not None:
            with open(p + ".attrs.tmp", "w") as f:
                json.dump(attrs, f)
            os.replace(p + ".attrs.tmp", p + ".attrs.json")

    def _read_array(self, node: str) -> np.ndarray:
        return np.load(self._path(node) + ".npy", allow_pickle=False)

    def write_tensor(self, tensor, node: str) -> None:
        """h5_io.tpp:243-291: the tensor's elements with its shape and element type as attributes."""
        a = np.ascontiguousarray(_to_numpy(tensor))
        self._write_array(node, a.reshape(-1), {"shape": list(a.shape), "type": a.dtype.str})

    def read_tensor(self, node: str) -> np.ndarray:
        """The stored tensor in its shape; the stored element type must be the one written."""
        a = self._read_array(node)
        with open(self._path(node) + ".attrs.json") as f:
            attrs = json.load(f)
        if a.dtype.str != attrs["type"]:
            raise TypeError(f"{node}: stored type {a.dtype.str} does not match its attribute {attrs['type']}")
        return a.reshape(attrs["shape"])

    # ---- Markov states ----------------------------------------------------------------------------------------------
    def write(self, state, node: str) -> None:
        """h5_io.tpp:68-167: the configuration's fields, actVal, acceptanceProbability, acceptanceRate, weights and
        markovTime of one Markov state under node (e.g. "markovChain/12")."""
        base = node.rstrip("/")
        for key, field in state.configuration.items():
            self.write_tensor(field, f"{base}/{key}")
        self._write_array(f"{base}/actVal", np.complex128(state.actionValue))
        self._write_array(f"{base}/acceptanceProbability", np.float64(state.acceptanceProbability))
        self._write_array(f"{base}/acceptanceRate", np.uint64(1 if state.accepted else 0))
        for key, w in state.weights.items():
            self._write_array(f"{base}/weights/{key}", np.complex128(w))
        self._write_array(f"{base}/markovTime", np.int32(state.markovTime))

    def read(self, state, node: str, markovTime: int | None = None):
        """h5_io.tpp:170-240 into `state` (whose configuration names the fields and whose weights name the keys to
        read): without markovTime the highest-numbered state under node. Returns state; raises if a dataset is
        missing or unreadable."""
        if markovTime is None:
            markovTime = self.getMinMaxConfigs(node)[1]
        base = f"{node.rstrip('/')}/{int(markovTime)}"
        state.markovTime = int(markovTime)
        state.configuration = Configuration({key: self.read_tensor(f"{base}/{key}")
                                             for key in state.configuration.keys()})
        state.actionValue = complex(self._read_array(f"{base}/actVal"))
        state.acceptanceProbability = float(self._read_array(f"{base}/acceptanceProbability"))
        state.weights = {key: complex(self._read_array(f"{base}/weights/{key}")) for key in state.weights}
        return state


def _to_numpy(x) -> np.ndarray:
    if hasattr(x, "detach"):  # a torch tensor, possibly on the GPU
        return x.detach().cpu().numpy()
    return np.asarray(x)
