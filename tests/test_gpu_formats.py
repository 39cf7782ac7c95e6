"""sample_write against files the reference's own CLI wrote for deterministic circuits (every noise
probability 0 or 1, so the bits do not depend on any random stream), in every result format and layout;
plus round trips of random data through the formats' published decoders."""

import os

import numpy as np
import pytest

import stim_gb300
from conftest import GOLDEN_DIR

pytestmark = pytest.mark.gpu

FMT_DIR = os.path.join(GOLDEN_DIR, "formats")


def cases():
    with open(os.path.join(FMT_DIR, "cases.txt")) as f:
        return [tuple(line.split()) for line in f if line.strip()]


def circuit(name):
    with open(os.path.join(FMT_DIR, name + ".stim")) as f:
        return stim_gb300.Circuit(f.read())


@pytest.mark.parametrize("case", cases(), ids=lambda c: c[0])
def test_sample_write_matches_reference_cli(case, tmp_path):
    fname, cname, fmt, layout = case
    c = circuit(cname)
    want = open(os.path.join(FMT_DIR, fname), "rb").read()
    out = tmp_path / "out"
    if cname == "meas":
        c.compile_sampler(seed=1).sample_write(128, filepath=str(out), format=fmt)
    elif layout in ("none", "append", "prepend"):
        c.compile_detector_sampler(seed=1).sample_write(128, filepath=out, format=fmt,
                                                        append_observables=layout == "append",
                                                        prepend_observables=layout == "prepend")
    else:
        obs = tmp_path / "obs"
        c.compile_detector_sampler(seed=1).sample_write(128, filepath=str(out), format=fmt,
                                                        obs_out_filepath=str(obs), obs_out_format=fmt)
        if layout == "obs":
            out = obs
    assert open(out, "rb").read() == want


def _decode(data, fmt, nbits, shots):
    """Decoders written from the format descriptions (dense bool matrix)."""
    out = np.zeros((shots, nbits), dtype=np.bool_)
    if fmt == "01":
        for s, line in enumerate(data.decode().split("\n")[:shots]):
            out[s] = [c == "1" for c in line]
    elif fmt == "b8":
        nb = (nbits + 7) // 8
        a = np.frombuffer(data, dtype=np.uint8).reshape(shots, nb)
        out[:] = np.unpackbits(a, axis=1, bitorder="little")[:, :nbits]
    elif fmt == "hits":
        for s, line in enumerate(data.decode().split("\n")[:shots]):
            for v in filter(None, line.split(",")):
                out[s, int(v)] = True
    elif fmt == "dets":
        for s, line in enumerate(data.decode().split("\n")[:shots]):
            parts = line.split()
            assert parts[0] == "shot"
            for v in parts[1:]:
                out[s, int(v[1:])] = True
    elif fmt == "r8":
        s, k, i = 0, 0, 0
        while s < shots:
            b = data[i]
            i += 1
            k += b
            if b == 255:
                continue
            if k < nbits:
                out[s, k] = True
                k += 1
            else:
                s, k = s + 1, 0
    elif fmt == "ptb64":
        words = np.frombuffer(data, dtype="<u8").reshape(shots // 64, nbits)
        for g in range(shots // 64):
            for m in range(nbits):
                w = int(words[g, m])
                for j in range(64):
                    out[g * 64 + j, m] = (w >> j) & 1
    return out


@pytest.mark.parametrize("fmt", ["01", "b8", "r8", "hits", "dets", "ptb64"])
def test_sample_write_round_trips_noisy_samples(fmt, tmp_path):
    from stim_gb300 import workloads

    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_x", 5, 5, 0.02))
    shots = 640
    path = tmp_path / "d"
    c.compile_detector_sampler(seed=3).sample_write(shots, filepath=path, format=fmt)
    want = c.compile_detector_sampler(seed=3).sample(shots)
    got = _decode(open(path, "rb").read(), fmt, c.num_detectors, shots)
    np.testing.assert_array_equal(got, want)


def test_sample_write_errors(tmp_path):
    c = circuit("det")
    s = c.compile_detector_sampler(seed=1)
    with pytest.raises(ValueError, match="Unrecognized output format"):
        s.sample_write(64, filepath=str(tmp_path / "x"), format="nope")
    with pytest.raises(ValueError, match="multiple of 64"):
        s.sample_write(65, filepath=str(tmp_path / "x"), format="ptb64")
    with pytest.raises(IndexError, match="Can't combine"):
        s.sample_write(64, filepath=str(tmp_path / "x"), append_observables=True,
                       obs_out_filepath=str(tmp_path / "y"))


@pytest.mark.parametrize("fmt", ["01", "b8", "r8", "hits", "dets", "ptb64"])
@pytest.mark.parametrize("family,d,p,shots", [("surface_code:rotated_memory_z", 25, 0.001, 4096),
                                              ("surface_code:rotated_memory_x", 11, 0.02, 8192)])
def test_device_formatted_files_equal_host_writer_at_scale(fmt, family, d, p, shots, tmp_path):
    # sample_write formats on the device; the same bits written by the host writer (write_shot_data_file, whose
    # files are pinned to the reference CLI's) must give the same bytes.
    from stim_gb300 import workloads

    c = stim_gb300.Circuit(workloads.code_circuit(family, d, d, p))
    D, O, M = c.num_detectors, c.num_observables, c.num_measurements
    out = tmp_path / "dev"
    c.compile_detector_sampler(seed=5).sample_write(shots, filepath=str(out), format=fmt, append_observables=True)
    bits = c.compile_detector_sampler(seed=5).sample(shots, bit_packed=True, append_observables=True)
    ref = tmp_path / "host"
    stim_gb300.write_shot_data_file(data=bits, path=str(ref), format=fmt, num_detectors=D, num_observables=O)
    assert open(out, "rb").read() == open(ref, "rb").read()
    mout = tmp_path / "mdev"
    c.compile_sampler(seed=6).sample_write(shots, filepath=str(mout), format=fmt)
    m = c.compile_sampler(seed=6).sample(shots, bit_packed=True)
    mref = tmp_path / "mhost"
    stim_gb300.write_shot_data_file(data=m, path=str(mref), format=fmt, num_measurements=M)
    assert open(mout, "rb").read() == open(mref, "rb").read()


@pytest.mark.parametrize("fmt", ["01", "b8", "r8", "hits", "dets", "ptb64"])
@pytest.mark.parametrize("layout", ["append", "prepend", "obs"])
def test_pipelined_chunks_equal_host_writer(fmt, layout, tmp_path):
    # Many small chunks through the two-slot file pipeline (and, for ptb64, the detector-major path), with every
    # observable layout, against the host writer on the same bits.
    from stim_gb300 import workloads

    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_z", 7, 7, 0.01))
    D, O = c.num_detectors, c.num_observables
    shots = 9 * 1024 + 64
    s = c.compile_detector_sampler(seed=11)
    s.set_chunk_shots(1024)
    out = tmp_path / "dev"
    if layout == "prepend" and fmt == "dets":
        # dets names prepended observables L0.. before the detectors, which the host writer's D-then-L rows cannot
        # express: compare against one chunk of the same device path (pinned to the reference CLI's file above).
        s.sample_write(shots, filepath=str(out), format=fmt, prepend_observables=True)
        c.compile_detector_sampler(seed=11).sample_write(shots, filepath=str(tmp_path / "h"), format=fmt,
                                                         prepend_observables=True)
    elif layout == "obs":
        obs = tmp_path / "obs"
        s.sample_write(shots, filepath=str(out), format=fmt, obs_out_filepath=str(obs), obs_out_format=fmt)
        d, o = c.compile_detector_sampler(seed=11).sample(shots, bit_packed=True, separate_observables=True)
        stim_gb300.write_shot_data_file(data=d, path=str(tmp_path / "h"), format=fmt, num_detectors=D)
        stim_gb300.write_shot_data_file(data=o, path=str(tmp_path / "ho"), format=fmt, num_observables=O)
        assert open(obs, "rb").read() == open(tmp_path / "ho", "rb").read()
    else:
        s.sample_write(shots, filepath=str(out), format=fmt, append_observables=layout == "append",
                       prepend_observables=layout == "prepend")
        bits = c.compile_detector_sampler(seed=11).sample(shots, bit_packed=True,
                                                          append_observables=layout == "append",
                                                          prepend_observables=layout == "prepend")
        stim_gb300.write_shot_data_file(data=bits, path=str(tmp_path / "h"), format=fmt, num_detectors=D,
                                        num_observables=O)
    assert open(out, "rb").read() == open(tmp_path / "h", "rb").read()
