"""Markov-chain files in NSL's H5IO node layout without HDF5 (nsl_gb300/markov_io.py) and HMC.generate's resume
logic (HMC.tpp:57-120), on the host: a stand-in HMC whose proposal is a deterministic host function drives
generate(), so no GPU is involved."""
import os

import numpy as np
import pytest

from nsl_gb300.configuration import Configuration
from nsl_gb300.hmc import HMC, MarkovState
from nsl_gb300.markov_io import MarkovChainFile


class HostHMC(HMC):
    """generate_ without the GPU, a deterministic function of the field: the proposal phi + 1 is accepted unless
    phi[0, 0] is a multiple of 3 (then the state is kept)."""

    def __init__(self):
        self.calls = 0

    def generate_(self, state):
        self.calls += 1
        phi0 = state.configuration["phi"]
        acc = int(round(phi0[0, 0].real)) % 3 != 0
        phi = phi0 + (1.0 if acc else 0.0)
        v = float(phi[0, 0].real)
        return MarkovState(Configuration({"phi": phi}), complex(phi.real.sum(), 0.5), 0.25 * v,
                           state.markovTime + 1, acc, {"logdetJ": complex(v, -v)})


def _start():
    phi = np.arange(12, dtype=np.complex128).reshape(3, 4) * (1 + 0.5j)
    return MarkovState(Configuration({"phi": phi}), complex(1.5, -2.0), 1.0, 1, True, {"logdetJ": 0j})


def test_state_round_trip_and_layout(tmp_path):
    f = MarkovChainFile(str(tmp_path / "chain"))
    s = HostHMC().generate_(_start())
    f.write(s, "markovChain/7")
    root = tmp_path / "chain" / "markovChain" / "7"
    for name in ("phi.npy", "phi.attrs.json", "actVal.npy", "acceptanceProbability.npy", "acceptanceRate.npy",
                 "markovTime.npy", os.path.join("weights", "logdetJ.npy")):
        assert (root / name).exists(), name
    assert np.load(root / "phi.npy").shape == (12,)  # flattened, the shape is an attribute (h5_io.tpp:243-291)
    r = f.read(_start(), "markovChain")
    assert r.markovTime == 7
    assert np.array_equal(r.configuration["phi"], s.configuration["phi"])
    assert r.actionValue == s.actionValue and r.acceptanceProbability == s.acceptanceProbability
    assert r.weights == s.weights
    assert int(np.load(root / "acceptanceRate.npy")) == int(s.accepted)
    assert f.getMinMaxConfigs("markovChain") == (7, 7)
    f.deleteData("markovChain/7")
    assert not f.exist("markovChain/7") and f.exist("markovChain")


def test_generate_writes_and_resumes(tmp_path):
    f = MarkovChainFile(str(tmp_path / "chain"))
    h = HostHMC()
    full = h.generate(_start(), 9, store=None)
    mc = HostHMC().generate(_start(), 5, store=f)
    assert f.getMinMaxConfigs("markovChain") == (0, 4)
    for n in range(5):
        assert np.array_equal(mc[n].configuration["phi"], full[n].configuration["phi"])
    # a longer run resumes from state 4: only states 5..8 are generated, and their fields equal the uninterrupted
    # chain's; as in the reference (h5_io.tpp:193) the resumed state's markovTime is its node number
    h2 = HostHMC()
    mc2 = h2.generate(_start(), 9, store=f)
    assert h2.calls == 4 and mc2[:4] == [None] * 4
    assert f.getMinMaxConfigs("markovChain") == (0, 8)
    for n in range(4, 9):
        assert np.array_equal(mc2[n].configuration["phi"], full[n].configuration["phi"])
        assert mc2[n].weights == full[n].weights
        assert mc2[n].markovTime == n


def test_generate_drops_an_unreadable_last_state(tmp_path):
    f = MarkovChainFile(str(tmp_path / "chain"))
    HostHMC().generate(_start(), 6, store=f)
    os.remove(tmp_path / "chain" / "markovChain" / "5" / "actVal.npy")  # state 5 half written
    h = HostHMC()
    mc = h.generate(_start(), 7, store=f)
    # state 5 is deleted, the run resumes from state 4 and regenerates 5 and 6
    assert h.calls == 2 and mc[4] is not None and mc[4].markovTime == 4
    assert f.getMinMaxConfigs("markovChain") == (0, 6)
    full = HostHMC().generate(_start(), 7)
    assert np.array_equal(mc[6].configuration["phi"], full[6].configuration["phi"])


def test_type_mismatch_and_bad_nodes_are_errors(tmp_path):
    f = MarkovChainFile(str(tmp_path / "chain"))
    f.write_tensor(np.ones((2, 2)), "t")
    np.save(str(tmp_path / "chain" / "t.npy"), np.ones(4, dtype=np.float32))  # element type changed behind its back
    with pytest.raises(TypeError):
        f.read_tensor("t")
    with pytest.raises(ValueError):
        f.exist("../outside")
    with pytest.raises(FileNotFoundError):
        f.getMinMaxConfigs("t_missing")


def test_generate_restarts_when_state_zero_is_unreadable(tmp_path):
    f = MarkovChainFile(str(tmp_path / "chain"))
    HostHMC().generate(_start(), 1, store=f)  # only state 0
    os.remove(tmp_path / "chain" / "markovChain" / "0" / "phi.npy")
    h = HostHMC()
    mc = h.generate(_start(), 3, store=f)
    assert h.calls == 2 and f.getMinMaxConfigs("markovChain") == (0, 2)
    assert np.array_equal(f.read(_start(), "markovChain", 0).configuration["phi"], _start().configuration["phi"])
    assert mc[0] is not None
