"""Run checkpoints on the host: big-wave's on-disk format (tests/golden/checkpoint_ref was written
by big-wave's RunCheckpoint, big-wave/checkpoint.py:83-208), transactional saves, and the
validation errors of load."""
import importlib
import json
import shutil
from pathlib import Path

import numpy as np
import pytest
import torch

GOLDEN = Path(__file__).resolve().parent / "golden"
FINGERPRINT = {"N": 64, "nx": 8, "ny": 8, "dtype": np.dtype(np.complex64).str, "wavelength": 6.2e-11,
               "z_detector": 1.5, "source_index": 3}


class Field:
    """Stand-in for a GpuVector on the CPU: a flat complex64 tensor in `vec`."""

    def __init__(self, n):
        self.vec = torch.zeros(n, dtype=torch.complex64)


@pytest.fixture(scope="module")
def ck():
    return importlib.import_module("3d_ravesim_gb300.checkpoint")


def test_reads_checkpoint_written_by_bigwave(ck, tmp_path):
    d = tmp_path / "ck"
    shutil.copytree(GOLDEN / "checkpoint_ref", d)
    u, U = Field(64), Field(64)
    state = ck.RunCheckpoint(d, FINGERPRINT).load(u, U)
    ref = np.load(GOLDEN / "checkpoint_ref_vectors.npy")
    np.testing.assert_array_equal(u.vec.numpy(), ref[0])
    np.testing.assert_array_equal(U.vec.numpy(), ref[1])
    assert state == ck.CheckpointState(0.125, 1, 10, 0, True, "element_slice")


def test_writes_bigwave_format(ck, tmp_path):
    ref = np.load(GOLDEN / "checkpoint_ref_vectors.npy")
    u, U = Field(64), Field(64)
    u.vec.copy_(torch.from_numpy(ref[0]))
    U.vec.copy_(torch.from_numpy(ref[1]))
    c = ck.RunCheckpoint(tmp_path, FINGERPRINT)
    c.save(u, U, current_z=0.125, element_index=1, slice_index=10, u_fourier_valid=True, stage="element_slice")
    ours = json.loads((tmp_path / "manifest.json").read_text())
    theirs = json.loads((GOLDEN / "checkpoint_ref" / "manifest.json").read_text())
    for m in (ours, theirs):
        for v in m["vectors"].values():
            v.pop("file")
    assert ours == theirs  # same keys, state, fingerprint and (same bytes) the same checksums
    assert sorted(p.name.split(".")[0] for p in tmp_path.glob("*.npy")) == ["spectrum", "u"]


def test_new_generation_replaces_old_and_complete_blocks_resume(ck, tmp_path):
    u, U = Field(64), Field(64)
    c = ck.RunCheckpoint(tmp_path, FINGERPRINT)
    for k in range(3):
        u.vec.fill_(k)
        c.save(u, U, current_z=0.1 * k, element_index=0, slice_index=5 * k, u_fourier_valid=True, stage="s")
    assert len(list(tmp_path.glob("u.*.npy"))) == 1 and not list(tmp_path.glob("*.part"))
    v = Field(64)
    assert c.load(v, Field(64)).slice_index == 10
    assert float(v.vec[0].real) == 2.0
    c.mark_complete()
    with pytest.raises(ValueError, match="not 'ready'"):
        c.load(Field(64), Field(64))


def test_load_rejects_wrong_fingerprint_and_corrupt_vectors(ck, tmp_path):
    d = tmp_path / "ck"
    shutil.copytree(GOLDEN / "checkpoint_ref", d)
    with pytest.raises(ValueError, match="fingerprint"):
        ck.RunCheckpoint(d, {**FINGERPRINT, "source_index": 4}).load(Field(64), Field(64))
    f = next(d.glob("u.*.npy"))
    raw = bytearray(f.read_bytes())
    raw[-1] ^= 1
    f.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        ck.RunCheckpoint(d, FINGERPRINT).load(Field(64), Field(64))


def test_cancel_token_interrupts_save(ck, tmp_path):
    class Token:
        is_set = True
    with pytest.raises(InterruptedError):
        ck.RunCheckpoint(tmp_path, FINGERPRINT, cancel_token=Token()).save(
            Field(64), Field(64), current_z=0.0, element_index=0, slice_index=0, u_fourier_valid=False, stage="s")
    assert not (tmp_path / "manifest.json").exists()


def test_interrupted_save_keeps_the_previous_generation_and_no_parts(ck, tmp_path):
    a = ck.RunCheckpoint(tmp_path, FINGERPRINT)
    u0, U0 = Field(64), Field(64)
    u0.vec = torch.randn(64, dtype=torch.complex64, generator=torch.Generator().manual_seed(4))
    a.save(u0, U0, current_z=0.5, element_index=1, slice_index=2, u_fourier_valid=True, stage="sample")
    before = sorted(p.name for p in tmp_path.iterdir())

    class Token:
        calls = 0

        def is_cancelled(self):  # lets the u vector be written, cancels before U
            Token.calls += 1
            return Token.calls > 1
    with pytest.raises(InterruptedError):
        ck.RunCheckpoint(tmp_path, FINGERPRINT, cancel_token=Token()).save(
            Field(64), Field(64), current_z=0.75, element_index=1, slice_index=3, u_fourier_valid=True, stage="s")
    assert sorted(p.name for p in tmp_path.iterdir()) == before
    u1, U1 = Field(64), Field(64)
    st = a.load(u1, U1)
    assert (st.current_z, st.slice_index) == (0.5, 2)
    assert np.array_equal(np.asarray(u1.vec), np.asarray(u0.vec))



def test_slice_checkpointer_saves_every_cadence_slice():
    ws = importlib.import_module("3d_ravesim_gb300.wavesim")
    saved = []

    class Recorder:
        def save(self, u, U, **state):
            saved.append((u, U, state))
    cb = ws._slice_checkpointer(Recorder(), "u", "U", 2)
    n = ws.CHECKPOINT_SLICE_CADENCE
    for k in range(1, 2 * n + 2):
        cb(k, 0.5 + 1e-6 * k)
    assert [s[2]["slice_index"] for s in saved] == [n, 2 * n]
    assert saved[0][:2] == ("u", "U")
    assert saved[0][2] == {"current_z": 0.5 + 1e-6 * n, "element_index": 2, "slice_index": n,
                           "u_fourier_valid": True, "stage": "element_slice"}
