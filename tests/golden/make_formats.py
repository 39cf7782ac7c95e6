"""Result-format fixtures written by the REFERENCE's own CLI (`stim detect` / `stim sample`) for
deterministic circuits (every noise probability 0 or 1), so the bits do not depend on its RNG.

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref
    python tests/golden/make_formats.py

It writes tests/golden/formats/<file> and cases.txt: one line per file, "<file> <circuit> <format>
<layout>", layout being none (detectors only), append (observables after the detectors), prepend
(observables first), sep (the detector file of a run whose observables went to <file minus .sep>.obs) or
obs (that observable file).  The CLI's dets output always names the observables too: first without
flags (layout prepend), last with --append_observables.
"""

import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
STIM = os.path.join(ROOT, "oracle", "_ref", "stim")
OUT = os.path.join(HERE, "formats")
FORMATS = ["01", "b8", "r8", "hits", "dets", "ptb64"]
SHOTS = 128

CIRCUITS = {
    # 300 detectors, some always firing, one always-flipped observable and one never-flipped one.
    "det": "X_ERROR(1) " + " ".join(str(q) for q in range(0, 300, 7)) + "\n"
           "M " + " ".join(str(q) for q in range(300)) + "\n"
           + "".join(f"DETECTOR rec[-{300 - q}]\n" for q in range(300))
           + "OBSERVABLE_INCLUDE(0) rec[-300]\nOBSERVABLE_INCLUDE(1) rec[-299]\n",
    # Measurements with a reference sample (X flips, an inverted target) and runs longer than 255.
    "meas": "X 0 5 600\nX_ERROR(1) 9 10\nM " + " ".join(str(q) for q in range(700)) + " !3\n",
}


def run(args):
    subprocess.run([STIM] + args, check=True, capture_output=True)


def main():
    os.makedirs(OUT, exist_ok=True)
    lines = []
    with tempfile.TemporaryDirectory() as td:
        for name, text in CIRCUITS.items():
            cpath = os.path.join(td, name + ".stim")
            with open(cpath, "w") as f:
                f.write(text)
            with open(os.path.join(OUT, name + ".stim"), "w") as f:
                f.write(text)
            for fmt in FORMATS:
                if name == "det":
                    base = f"det.{fmt}"
                    common = ["detect", "--in", cpath, "--shots", str(SHOTS), "--out_format", fmt]
                    if fmt == "dets":
                        # Without flags the CLI's dets output names the observables first.
                        run(common + ["--out", os.path.join(OUT, base)])
                        lines.append(f"{base} det {fmt} prepend")
                        run(common + ["--out", os.path.join(OUT, base + ".append"), "--append_observables"])
                        lines.append(f"{base}.append det {fmt} append")
                        continue
                    run(common + ["--out", os.path.join(OUT, base)])
                    lines.append(f"{base} det {fmt} none")
                    run(common + ["--out", os.path.join(OUT, base + ".append"), "--append_observables"])
                    lines.append(f"{base}.append det {fmt} append")
                    run(common + ["--out", os.path.join(OUT, base + ".sep"), "--obs_out",
                                  os.path.join(OUT, base + ".obs"), "--obs_out_format", fmt])
                    lines.append(f"{base}.sep det {fmt} sep")
                    lines.append(f"{base}.obs det {fmt} obs")
                else:
                    run(["sample", "--in", cpath, "--shots", str(SHOTS), "--out_format", fmt, "--out",
                         os.path.join(OUT, f"meas.{fmt}")])
                    lines.append(f"meas.{fmt} meas {fmt} none")
    with open(os.path.join(OUT, "cases.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
