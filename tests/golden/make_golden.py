"""Generate the golden fixtures of this directory.

known_answers.json -- the known answers of the reference's NESL test suite
    (nesl/neslsrc/test.nesl, line numbers in each case's "source"), restated
    as the CVL primitive calls vinterp makes for them.  Strings are vectors
    of character codes, booleans are cvl_bool 0/1, and scans are the raw
    exclusive scans (the NESL tests combine max_scan/min_scan with the input
    elementwise; the scan values here are what those tests imply).

serial_cvl.npz -- seeded random inputs and the outputs of the reference's
    own serial CVL, compiled from its sources by `make -C oracle ref`
    (with -Di386=1, see oracle/Makefile).  Run where that library exists:

        make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

INT_MIN, INT_MAX = -(2 ** 31), 2 ** 31 - 1
F36 = float(np.float32(1e36))


def s(txt):
    return [ord(ch) for ch in txt]


def known_answers():
    C = []

    def add(what, source, fn, call, args, want):
        C.append(dict(what=what, source=f"nesl/neslsrc/test.nesl:{source}", fn=fn, call=call,
                      args=args, want=want))

    add("plus_scan", "62-63", "add_suz", "scan_u", [[2, -4, 3, 3]], [0, 2, -2, 1])
    add("float plus_scan", "65-66", "add_sud", "scan_u", [[2.0, -3.0, 3.0]], [0.0, 2.0, -1.0])
    add("mult_scan", "68-69", "mul_suz", "scan_u", [[2, -3, 3]], [1, 2, -6])
    add("float mult_scan", "71-72", "mul_sud", "scan_u", [[2.0, -3.0, 3.0]], [1.0, 2.0, -6.0])
    add("max_val", "74-75", "max_ruz", "reduce_u", [[-5, 23, -100, 7, 0, -2]], 23)
    add("min_val", "77-78", "min_ruz", "reduce_u", [[-5, 23, -100, 7000, 0, -2]], -100)
    add("max_scan", "80-83", "max_suz", "scan_u", [[-5, 8, 1]], [INT_MIN, -5, 8])
    add("float max_scan", "85-88", "max_sud", "scan_u", [[-5.0, 8.0, 1.0]], [-F36, -5.0, 8.0])
    add("min_scan", "90-93", "min_suz", "scan_u", [[5, -8, -1]], [INT_MAX, 5, -8])
    add("float min_scan", "95-98", "min_sud", "scan_u", [[5.0, -8.0, -1.0]], [F36, 5.0, -8.0])
    add("or_scan", "100-102", "ior_sub", "scan_u", [[0, 0, 0, 1, 0, 0, 0]], [0, 0, 0, 0, 1, 1, 1])
    add("and_scan", "104-106", "and_sub", "scan_u", [[1, 1, 1, 0, 1, 0, 1]], [1, 1, 1, 1, 0, 0, 0])
    add("xor_scan", "108-110", "xor_sub", "scan_u", [[0, 1, 0, 1, 0, 0, 0]], [0, 0, 1, 1, 0, 0, 0])
    add("int or_scan", "112-113", "ior_suz", "scan_u", [[6, 1, 32768, 63, 32704, 99]],
        [0, 6, 7, 32775, 32831, 65535])
    add("int and_scan", "115-116", "and_suz", "scan_u", [[32767, 29, 11, 9, 0, 65535]],
        [-1, 32767, 29, 9, 9, 0])
    add("int xor_scan", "118-120", "xor_suz", "scan_u", [[0, 0, 0, 32767, 32767, 32767, 3, 0, 3]],
        [0, 0, 0, 0, 32767, 0, 32767, 32764, 32764])
    add("permute", "122-124", "smp_puz", "smp_u", [s("mowtab"), [2, 1, 0, 5, 4, 3]], s("wombat"))
    add("bool permute", "133-135", "smp_pub", "smp_u", [[0, 0, 1, 1, 1, 1], [2, 4, 0, 1, 3, 5]],
        [1, 1, 0, 1, 0, 1])
    add("put", "137-139", "dpe_puz", "dpe_u", [s("mowtab"), [2, 1, 0, 6, 5, 4], s("testing it")],
        s("womtbat it"))
    add("bool put", "141-143", "dpe_pub", "dpe_u", [[0, 1, 1, 0], [4, 0, 5, 1], [0, 0, 0, 1, 0, 0]],
        [1, 0, 0, 1, 0, 1])
    add("cond_put", "145-147", "dfp_puz", "dfp_u",
        [s("mowtab"), [2, 1, 0, 6, 5, 4], [1, 1, 1, 0, 0, 0], s("testing it")], s("womting it"))
    add("bool cond_put", "149-151", "dfp_pub", "dfp_u",
        [[0, 1, 1, 1], [5, 2, 2, 4], [1, 1, 0, 0], [1, 1, 0, 0, 1, 0, 0, 0]],
        [1, 1, 1, 0, 1, 0, 0, 0])
    get_idx = list(range(17, 99, 11))
    add("float get", "153-155", "bck_pud", "bck_u", [[float(j) for j in range(100, 200)], get_idx],
        [117.0, 128.0, 139.0, 150.0, 161.0, 172.0, 183.0, 194.0])
    add("bool get", "157-159", "bck_pub", "bck_u", [[int(j % 3 == 0) for j in range(100, 200)], get_idx],
        [1, 0, 0, 1, 0, 0, 1, 0])
    add("get", "161-163", "bck_puz", "bck_u", [s("testing it"), [3, 4, 1]], s("tie"))
    add("pack", "165-166", "pk2_luz", "pack_u", [s("the horse"), [1, 0, 1, 1, 0, 0, 1, 1, 0]], s("te rs"))
    add("bool pack", "168-169", "pk2_lub", "pack_u",
        [[1, 0, 1, 0, 1, 1, 1, 0, 0], [1, 0, 1, 1, 0, 0, 1, 1, 0]], [1, 1, 0, 1, 0])
    add("float pack", "171-173", "pk2_lud", "pack_u",
        [[0.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0], [1, 0, 1, 0, 1, 1, 0, 1]], [0.0, 2.0, 4.0, 5.0, 7.0])
    add("trunc", "178", "trn_wud", "ew1", [[3.2]], [3])
    add("floor", "180", "flr_wud", "ew1", [[-3.2]], [-4])
    add("ceil", "182", "cei_wud", "ew1", [[-3.2]], [-3])
    add("round", "184", "rou_wud", "ew1", [[4.6]], [5])
    add("seg int dist", "344-345", "dis_vez", "dis_e", [s("af"), [1, 2]], s("aff"))
    add("seg int dist (zero len)", "346-347", "dis_vez", "dis_e", [s("ahf"), [1, 0, 2]], s("aff"))
    add("seg int sum", "348-349", "add_rez", "reduce_e", [[2, 3, 3, 2], [3, 1]], [8, 2])
    add("seg int sum (zero len)", "350-351", "add_rez", "reduce_e", [[2, 3, 3, 2], [3, 0, 1]], [8, 0, 2])
    key = [10, -5, 0, 10, -10, 100, 10]
    add("int rank", "627-628", "rku_luz", "rank_u", [key], [3, 1, 2, 4, 0, 6, 5])
    add("int rank_down", "629-630", "rkd_luz", "rank_u", [key], [1, 5, 4, 2, 6, 0, 3])
    add("float rank", "631-633", "rku_lud", "rank_u", [[float(k) for k in key]], [3, 1, 2, 4, 0, 6, 5])
    add("float rank_down", "634-636", "rkd_lud", "rank_u", [[float(k) for k in key]], [1, 5, 4, 2, 6, 0, 3])
    return dict(note=__doc__.split("\n\n")[1], cases=C)


def serial_vectors():
    from neslgpu_gb300 import ops
    from neslgpu_gb300 import workloads as W
    from oracle.oracle import HostRunner, load_reference
    ref = load_reference()
    if ref is None:
        raise SystemExit("build the reference serial CVL first: make -C oracle ref")
    R = HostRunner(ref)
    r = W.rng(2024)
    n = 3000
    xi = W.int32_uniform(r, n)
    xd = W.float64_normal(r, n)
    lens = W.with_empty(r, W.geometric_lengths(r, n, 24), 0.2)
    perm = W.permutation(r, n)
    sperm = W.seg_permutation(r, lens)
    flags = r.integers(0, 2, size=n).astype(np.int32)
    ties = (xi % 17).astype(np.int32)
    tied_d = np.round(xd * 3) / 3
    out = dict(xi=xi, xd=xd, lens=lens, perm=perm, sperm=sperm, flags=flags, ties=ties, tied_d=tied_d)
    out["add_sez"] = ops.scan_e(R, "add_sez", xi, lens)
    out["add_sed"] = ops.scan_e(R, "add_sed", xd, lens)
    out["max_sed"] = ops.scan_e(R, "max_sed", xd, lens)
    out["add_red"] = ops.reduce_e(R, "add_red", xd, lens)
    out["max_rez"] = ops.reduce_e(R, "max_rez", xi, lens)
    out["min_red"] = ops.reduce_e(R, "min_red", xd, lens)
    out["pk2_luz"] = ops.pack_u(R, "pk2_luz", xi, flags)
    out["pk1_lev"] = ops.pk1_e(R, flags, lens)
    out["smp_puz"] = ops.smp_u(R, "smp_puz", xi, perm)
    out["smp_ped"] = ops.smp_e(R, "smp_ped", xd, sperm, lens)
    out["bck_pez"] = ops.bck_e(R, "bck_pez", xi, sperm, lens, lens)
    out["rku_luz"] = ops.rank_u(R, "rku_luz", xi)
    out["rkd_luz"] = ops.rank_u(R, "rkd_luz", ties)
    out["rku_lud"] = ops.rank_u(R, "rku_lud", xd)
    out["rkd_lud"] = ops.rank_u(R, "rkd_lud", tied_d)
    out["rku_lez"] = ops.rank_e(R, "rku_lez", ties, lens)
    out["rkd_led"] = ops.rank_e(R, "rkd_led", tied_d, lens)
    return out


if __name__ == "__main__":
    (HERE / "known_answers.json").write_text(json.dumps(known_answers(), indent=1) + "\n")
    np.savez_compressed(HERE / "serial_cvl.npz", **serial_vectors())
    print("wrote", HERE / "known_answers.json", HERE / "serial_cvl.npz")
