"""Golden vectors produced by the reference's own serial CVL
(tests/golden/make_golden.py): the oracle must reproduce them bit for bit,
and the GPU library within the parity tolerances."""
from pathlib import Path

import numpy as np
import pytest

from cases import compare, seg_abs_prefix, seg_abs_total
from neslgpu_gb300 import ops

G = dict(np.load(Path(__file__).parent / "golden" / "serial_cvl.npz"))


def _results(R):
    g = G
    return {
        "add_sez": ops.scan_e(R, "add_sez", g["xi"], g["lens"]),
        "add_sed": ops.scan_e(R, "add_sed", g["xd"], g["lens"]),
        "max_sed": ops.scan_e(R, "max_sed", g["xd"], g["lens"]),
        "add_red": ops.reduce_e(R, "add_red", g["xd"], g["lens"]),
        "max_rez": ops.reduce_e(R, "max_rez", g["xi"], g["lens"]),
        "min_red": ops.reduce_e(R, "min_red", g["xd"], g["lens"]),
        "pk2_luz": ops.pack_u(R, "pk2_luz", g["xi"], g["flags"]),
        "pk1_lev": ops.pk1_e(R, g["flags"], g["lens"]),
        "smp_puz": ops.smp_u(R, "smp_puz", g["xi"], g["perm"]),
        "smp_ped": ops.smp_e(R, "smp_ped", g["xd"], g["sperm"], g["lens"]),
        "bck_pez": ops.bck_e(R, "bck_pez", g["xi"], g["sperm"], g["lens"], g["lens"]),
        "rku_luz": ops.rank_u(R, "rku_luz", g["xi"]),
        "rkd_luz": ops.rank_u(R, "rkd_luz", g["ties"]),
        "rku_lud": ops.rank_u(R, "rku_lud", g["xd"]),
        "rkd_lud": ops.rank_u(R, "rkd_lud", g["tied_d"]),
        "rku_lez": ops.rank_e(R, "rku_lez", g["ties"], g["lens"]),
        "rkd_led": ops.rank_e(R, "rkd_led", g["tied_d"], g["lens"]),
    }


def test_golden_oracle(oracle):
    for k, v in _results(oracle).items():
        compare("exact", v, G[k])


@pytest.mark.gpu
def test_golden_gpu(gpu):
    ctx = {"add_sed": seg_abs_prefix(G["xd"], G["lens"]), "add_red": seg_abs_total(G["xd"], G["lens"])}
    for k, v in _results(gpu).items():
        compare("sum" if k in ctx else "exact", v, G[k], ctx.get(k))
