"""The host side of the boundary against the reference's own command-line tool, on seeded random inputs (CPU; skipped
where the reference has not been built into oracle/_ref by `make -C oracle ref`):

* circuit texts: accepted / rejected as `stim sample` and `stim detect` accept them, with the same measurement count;
* reference samples: equal to the reference's, read back through `stim m2d` of an all-zero record with one detector
  per measurement (multi-target measurements, resets, pair measurements, products and feedback on entangled qubits);
* detector error models: accepted / rejected as `stim sample_dem` accepts them, with the same detector and observable
  counts;
* result files: this package's reader reads what `stim convert` writes, and its writer writes the same bytes;
  malformed files are rejected exactly when `stim convert` rejects them.

The reference is run as the checker only; nothing here is on the product path."""

import os
import random
import subprocess

import numpy as np
import pytest

import stim_gb300

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "stim")

pytestmark = pytest.mark.skipif(not os.path.isfile(REF), reason="the reference CLI is not built (make -C oracle ref)")


def ref(args, stdin=None):
    return subprocess.run([REF] + args, capture_output=True, text=True, errors="replace", input=stdin)


def ours_accepts(text, mode):
    try:
        c = stim_gb300.Circuit(text)
        c.reference_sample()
        c.program_info(mode)
        return c
    except (ValueError, IndexError):
        return None


def random_target(r):
    k = r.random()
    q = r.choice([0, 1, 2, 3, 5])
    if k < 0.5:
        return str(q)
    if k < 0.6:
        return "!" + str(q)
    if k < 0.7:
        return f"rec[-{r.choice([1, 2, 3, 100])}]"
    if k < 0.75:
        return f"sweep[{r.choice([0, 3])}]"
    if k < 0.88:
        return r.choice("XYZ") + str(q)
    if k < 0.93:
        return f"{r.choice('XYZ')}{q}*{r.choice('XYZ')}{(q + 1) % 6}"
    return r.choice(["*", "-1", "a", "rec[0]", "X", "!rec[-1]", "2.5"])


def random_text(r):
    gates = ["H", "S", "CX", "CZ", "CY", "XCZ", "SWAP", "ISWAP", "M", "MX", "MY", "MR", "MRX", "R", "RX", "MPP", "SPP",
             "MXX", "MYY", "MZZ", "MPAD", "X_ERROR", "DEPOLARIZE1", "DEPOLARIZE2", "PAULI_CHANNEL_1", "E", "DETECTOR",
             "OBSERVABLE_INCLUDE", "TICK", "QUBIT_COORDS", "HERALDED_ERASE", "I", "SQRT_XX", "C_XYZ"]
    args = ["", "", "(0.1)", "(0)", "(1)", "()", "(-0.1)", "(1.5)", "(0.1, 0.2)", "(0.1,0.2,0.3)", "(nan)", "(2)"]
    lines, depth = [], 0
    for _ in range(r.randint(1, 8)):
        k = r.random()
        if k < 0.08:
            lines.append(f"REPEAT {r.choice([0, 1, 2, 3])} {{")
            depth += 1
        elif k < 0.14 and depth:
            lines.append("}")
            depth -= 1
        else:
            g = r.choice(gates)
            lines.append(f"{g}{r.choice(args)} " + " ".join(random_target(r) for _ in range(r.choice([0, 1, 2, 2, 4]))))
    return "\n".join(lines + ["}"] * depth)


@pytest.mark.parametrize("cmd,mode", [("sample", "measurements"), ("detect", "detections")])
def test_circuit_acceptance_matches_reference_cli(cmd, mode, tmp_path):
    r = random.Random(2024 if cmd == "sample" else 2025)
    path = tmp_path / "c.stim"
    for _ in range(150):
        text = random_text(r)
        path.write_text(text)
        p = ref([cmd, "--shots", "1", "--in", str(path), "--out_format", "01"])
        c = ours_accepts(text, mode)
        assert (p.returncode == 0) == (c is not None), (text, p.stderr[:200])
        if c is not None and cmd == "sample":
            assert len(p.stdout.strip()) == c.num_measurements, text


def random_valid_circuit(r, n):
    one = ["H", "S", "S_DAG", "SQRT_X", "H_YZ", "C_XYZ", "X", "Y", "H_XY"]
    two = ["CX", "CY", "CZ", "XCY", "YCZ", "SWAP", "ISWAP", "CXSWAP", "SQRT_XX", "SQRT_ZZ_DAG"]
    lines = ["M 0"]
    for _ in range(r.randint(4, 14)):
        qs = r.sample(range(n), n)
        m = r.randint(1, n)
        k = r.randrange(7)
        if k == 0:
            lines.append(f"{r.choice(one)} " + " ".join(map(str, qs[:m])))
        elif k == 1:
            lines.append(f"{r.choice(two)} " + " ".join(map(str, qs[:2 * max(1, m // 2)])))
        elif k == 2:
            g = r.choice(["M", "MX", "MY", "MR", "MRX", "MRY"])
            lines.append(f"{g} " + " ".join(("!" if r.random() < 0.2 else "") + str(q) for q in qs[:m]))
        elif k == 3:
            lines.append(f"{r.choice(['R', 'RX', 'RY'])} " + " ".join(map(str, qs[:m])))
        elif k == 4:
            tgts = qs[:2 * max(1, m // 2)] + r.sample(range(n), 2)  # a repeated qubit starts a new run
            lines.append(f"{r.choice(['MXX', 'MYY', 'MZZ'])} " + " ".join(map(str, tgts)))
        elif k == 5:
            prods = ["*".join(f"{r.choice('XYZ')}{q}" for q in r.sample(range(n), r.randint(1, min(3, n))))
                     for _ in range(r.randint(1, 3))]
            lines.append(f"{r.choice(['MPP', 'MPP', 'SPP', 'SPP_DAG'])} " + " ".join(prods))
        else:
            lines.append(f"{r.choice(['CX', 'CY', 'CZ'])} rec[-1] {qs[0]}")
    return "\n".join(lines)


def test_reference_samples_match_reference_cli(tmp_path):
    r = random.Random(7)
    path = tmp_path / "c.stim"
    for _ in range(120):
        text = random_valid_circuit(r, r.randint(2, 8))
        c = stim_gb300.Circuit(text)
        M = c.num_measurements
        path.write_text(text + "\n" + "\n".join(f"DETECTOR rec[-{M - k}]" for k in range(M)))
        p = ref(["m2d", "--in_format", "01", "--out_format", "01", "--circuit", str(path)], stdin="0" * M + "\n")
        assert p.returncode == 0, p.stderr
        want = np.array([ch == "1" for ch in p.stdout.strip()[-M:]])
        np.testing.assert_array_equal(c.reference_sample(), want, err_msg=text)


def random_dem(r):
    def tgt():
        k = r.random()
        if k < 0.5:
            return f"D{r.choice([0, 1, 5, 100])}"
        if k < 0.75:
            return f"L{r.choice([0, 1, 3])}"
        if k < 0.85:
            return "^"
        return r.choice(["D-1", "X0", "L", "5", "d3"])
    lines = []
    for _ in range(r.randint(1, 7)):
        k = r.random()
        if k < 0.5:
            p = r.choice(["0", "0.1", "1", "-0.1", "1.5", "", "0.1,0.2", "\t0.2 "])
            lines.append(f"error{r.choice(['', '[t]'])}{r.choice(['', '', ' '])}({p})" + r.choice([" ", "", "  "])
                         + " ".join(tgt() for _ in range(r.randint(0, 4))))
        elif k < 0.65:
            lines.append(f"detector{r.choice(['', '(1,2)', '(,)'])} " + " ".join(tgt() for _ in range(r.randint(0, 2))))
        elif k < 0.75:
            lines.append("logical_observable " + " ".join(tgt() for _ in range(r.randint(0, 2))))
        elif k < 0.85:
            lines.append(f"shift_detectors{r.choice(['', '(1)'])} {r.choice(['0', '3', '-1', ''])}")
        elif k < 0.93:
            lines.append(f"repeat {r.choice(['0', '2', ''])} {{")
        else:
            lines.append(r.choice(["}", "detector D0}", "error(0.1) D0 }"]))
    return "\n".join(lines)


def test_detector_error_models_match_reference_cli(tmp_path):
    r = random.Random(11)
    path, out, obs = tmp_path / "m.dem", tmp_path / "d", tmp_path / "o"
    for _ in range(200):
        text = random_dem(r)
        path.write_text(text)
        p = ref(["sample_dem", "--shots", "1", "--in", str(path), "--out", str(out), "--out_format", "01",
                 "--obs_out", str(obs), "--obs_out_format", "01"])
        try:
            m = stim_gb300.DetectorErrorModel(text)
        except (ValueError, IndexError):
            m = None
        assert (p.returncode == 0) == (m is not None), (text, p.stderr[:200])
        if m is not None:
            assert len(out.read_text().split("\n")[0]) == m.num_detectors, text
            assert len(obs.read_text().split("\n")[0]) == m.num_observables, text


def test_result_files_match_reference_convert(tmp_path):
    r = random.Random(13)
    fmts = ["01", "b8", "r8", "hits", "dets", "ptb64"]
    a, b, c = tmp_path / "a", tmp_path / "b", tmp_path / "c"
    for it in range(120):
        nm = r.choice([1, 7, 8, 9, 63, 64, 65, 300])
        shots = r.choice([64, 128]) if r.random() < 0.5 else r.randint(1, 70)
        data = np.random.default_rng(it).random((shots, nm)) < r.choice([0.0, 0.02, 0.4, 1.0])
        fin, fout = r.choice(fmts), r.choice(fmts[:5])  # the reference writes ptb64 only from whole tables
        if fin == "ptb64" and shots % 64:
            continue
        counts = {"num_measurements": nm, "num_detectors": 0, "num_observables": 0}
        if "dets" in (fin, fout) and r.random() < 0.5:
            d = r.randint(0, nm)
            counts = {"num_measurements": 0, "num_detectors": d, "num_observables": nm - d}
        kw = {k: v for k, v in counts.items() if v} or {"num_measurements": nm}
        stim_gb300.write_shot_data_file(data=data, path=str(a), format=fin, **kw)
        p = ref(["convert", "--in", str(a), "--in_format", fin, "--out", str(b), "--out_format", fout] +
                [x for k, v in counts.items() for x in (f"--{k}", str(v))])
        assert p.returncode == 0, p.stderr
        back = stim_gb300.read_shot_data_file(path=str(b), format=fout, **kw)
        np.testing.assert_array_equal(back, data)
        stim_gb300.write_shot_data_file(data=data, path=str(c), format=fout, **kw)
        assert c.read_bytes() == b.read_bytes(), (fin, fout, nm, shots, counts)


def test_malformed_result_files_read_like_reference_convert(tmp_path):
    # Random, often malformed files in every format: accepted or rejected as `stim convert` accepts them, and when
    # accepted, read as the same bits.
    r = random.Random(17)
    a, b = tmp_path / "a", tmp_path / "b"

    def make(fmt, nm):
        if fmt == "01":
            lines = ["".join(r.choice("01") for _ in range(nm + r.choice([0, 0, 0, -1, 1])))
                     for _ in range(r.randint(0, 4))]
            text = "\n".join(lines) + r.choice(["\n", "", "\n\n", "\r\n"])
            return (text.replace("1", "2", 1) if r.random() < 0.1 else text).encode()
        if fmt == "b8":
            return bytes(r.randrange(256) for _ in range(r.randint(0, 3 * ((nm + 7) // 8) + 1)))
        if fmt == "r8":
            return bytes(r.choice([0, 1, 2, 5, 255, nm]) % 256 for _ in range(r.randint(0, 8)))
        if fmt == "hits":
            lines = [",".join(str(r.randrange(nm + 2)) for _ in range(r.randint(0, 3))) for _ in range(r.randint(0, 3))]
            return ("\n".join(lines) + r.choice(["\n", ""])).encode()
        if fmt == "dets":
            lines = ["shot" + "".join(f" {r.choice('MDL')}{r.randrange(nm + 1)}" for _ in range(r.randint(0, 3)))
                     for _ in range(r.randint(0, 3))]
            return ("\n".join(lines) + r.choice(["\n", ""])).encode()
        return bytes(r.randrange(256) for _ in range(8 * nm * r.randint(0, 2) + r.choice([0, 0, 3])))

    for _ in range(300):
        fmt = r.choice(["01", "b8", "r8", "hits", "dets", "ptb64"])
        nm = r.choice([1, 3, 8, 9, 16, 17])
        a.write_bytes(make(fmt, nm))
        p = ref(["convert", "--in", str(a), "--in_format", fmt, "--out", str(b), "--out_format", "01",
                 "--num_measurements", str(nm), "--num_detectors", "0", "--num_observables", "0"])
        try:
            got = stim_gb300.read_shot_data_file(path=str(a), format=fmt, num_measurements=nm)
        except (ValueError, IndexError):
            got = None
        assert (p.returncode == 0) == (got is not None), (fmt, nm, a.read_bytes()[:60], p.stderr[:100])
        if got is not None:
            rows = [[ch == "1" for ch in ln] for ln in b.read_text().split("\n") if ln]
            want = np.array(rows, dtype=np.bool_).reshape(-1, nm) if rows else np.zeros((0, nm), dtype=np.bool_)
            np.testing.assert_array_equal(got, want)
