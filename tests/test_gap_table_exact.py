"""The contract's geometric skipping (stim_gb300/csrc/gfs_contract.h, shared by the kernels and the oracle) against
the geometric distribution it restates (the reference's RareErrorIterator, src/stim/util_bot/probability_util.h:
33-71: the gap before the next hit is k with probability p (1-p)^k).  Exact checks on the host, no sampling:

* the threshold table T[k] is 2^32 (1-p)^k to within 2^-20 relative (or one unit of 2^32) for k up to the
  segment's 2,048 trials, at p from 1e-6 to 0.99;
* the gap lookup returns max{k : u < T[k]} for every draw u and every starting guess (the property the kernels'
  float estimate relies on), checked by brute force on seeded draws;
* a draw below T[room] leaves the segment, any other lands a hit inside it."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "stim_gb300", "csrc")

PROGRAM = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "gfs_contract.h"
static uint64_t s = 88172645463325252ull;
static uint32_t next(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return (uint32_t)(s >> 11); }
int main(void) {
    static uint32_t T[GFS_SEG_TRIALS + 1];
    const double ps[] = {1e-6, 1e-4, 1e-3, 0.01, 0.1, 0.3, 0.5, 0.9, 0.99};
    double worst = 0;
    long bad_fixup = 0, bad_leave = 0;
    for (unsigned i = 0; i < sizeof(ps) / sizeof(ps[0]); i++) {
        const double p = ps[i];
        gfs_build_gap_table(p, T);
        for (int k = 1; k <= GFS_SEG_TRIALS; k++) {
            const double exact = ldexp(pow(1.0 - p, k), 32);
            const double err = fabs((double)T[k] - exact);
            const double rel = err / (exact > 1.0 ? exact : 1.0);
            if (err > 1.0 && rel > worst) worst = rel;
        }
        for (int t = 0; t < 20000; t++) {
            const uint32_t u = next();
            const int maxk = 1 + (int)(next() % GFS_SEG_TRIALS) - 1;
            int want = 0;
            for (int k = 1; k <= maxk; k++) if (u < T[k]) want = k;
            const int est = (int)(next() % (GFS_SEG_TRIALS + 40)) - 20;
            if ((int)gfs_gap_fixup(u, T, est, maxk) != want) bad_fixup++;
            const int room = 1 + (int)(next() % GFS_SEG_TRIALS);
            const int hit = gfs_hit_after_draw(u, T, gfs_inv_c(p), -1, room);
            if ((u < T[room]) != (hit < 0) || (hit >= room)) bad_leave++;
        }
    }
    printf("%.3e %ld %ld\n", worst, bad_fixup, bad_leave);
    return 0;
}
"""


def test_gap_table_and_lookup_are_exact(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src, exe = tmp_path / "gap.c", tmp_path / "gap"
    src.write_text(PROGRAM)
    subprocess.run([cc, "-std=c11", "-O1", "-I", CSRC, str(src), "-o", str(exe), "-lm"], check=True)
    worst, bad_fixup, bad_leave = subprocess.run([str(exe)], capture_output=True, text=True,
                                                 check=True).stdout.split()
    assert float(worst) < 2 ** -20
    assert int(bad_fixup) == 0
    assert int(bad_leave) == 0
