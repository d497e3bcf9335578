"""Generate the committed golden vectors in tests/golden/golden_lup.npz.

Run where the reference sources are present, after building the reference's own
float32 CPU determinant into oracle/_ref:

    make -C oracle ref REF=<reference checkout>/LU-fqhe
    python tests/golden/make_golden.py --ref-dir <reference checkout>/LU-fqhe

Inputs are seeded and stored explicitly, so the fixture does not depend on any
generator:
  * gauss_n{2,3,4,8,16}: complex Gaussian, Re/Im ~ N(0, 1/2)
  * lll_n24: lowest-Landau-level orbital matrices, z ~ CN(0, 24)
  * ref_fixture: 16 matrices of the reference's shipped input file
    LU-fqhe/inc/1000_16x16.bin (its only fixture; it has no expected outputs)
  * ref_fixture_all: all 1000 matrices of that file, as complex64
Outputs stored per set: the reference's float32 determinant (its bits) and a
64-bit digest of the factors it leaves in place; the FP64 restatement's
log|det|, phase, parity and pivot sequence (oracle literal mode); and the
double-double truth.
"""
import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import lufqhe_oracle as orc  # noqa: E402


def gauss(rng, b, n):
    return (rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n))) / np.sqrt(2)


def lll(rng, b, n):
    z = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))) * np.sqrt(n / 2)
    return z[:, :, None] ** np.arange(n)[None, None, :] * np.exp(-np.abs(z) ** 2 / 4)[:, :, None]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", required=True,
                    help="the reference's LU-fqhe directory (holds inc/1000_16x16.bin)")
    args = ap.parse_args()
    if not orc.ref_available():
        raise SystemExit("build oracle/_ref first (make -C oracle ref REF=...)")
    fixture = Path(args.ref_dir) / "inc" / "1000_16x16.bin"
    raw = np.fromfile(fixture, dtype=np.float32).view(np.complex64).reshape(-1, 16, 16)
    rng = np.random.default_rng(20130307)
    sets = {}
    for n in (2, 3, 4, 8, 16):
        sets[f"gauss_n{n}"] = gauss(rng, 24, n)
    sets["lll_n24"] = lll(rng, 16, 24)
    sets["ref_fixture"] = raw[:16].astype(np.complex128)
    out = {}
    for name, A in sets.items():
        A = A.astype(np.complex64).astype(np.complex128)  # exactly representable in float32
        res = orc.lup_det(A, arith=orc.ARITH_LITERAL)
        la_dd, ph_dd, _ = orc.logdet_dd(A)
        det32, fac32 = orc.ref_factor_f32(A.astype(np.complex64))
        out[f"{name}/A"] = A
        out[f"{name}/ref_det_f32"] = det32
        out[f"{name}/ref_factor_digest"] = orc.factor_digests(fac32)
        out[f"{name}/logabs"] = res["logabs"]
        out[f"{name}/phase"] = res["phase"]
        out[f"{name}/parity"] = res["parity"]
        out[f"{name}/piv"] = res["piv"]
        out[f"{name}/logabs_dd"] = la_dd
        out[f"{name}/phase_dd"] = ph_dd
    # the whole fixture file, as the reference reads it (complex64)
    det32, fac32 = orc.ref_factor_f32(raw)
    A = raw.astype(np.complex128)
    la_dd, ph_dd, _ = orc.logdet_dd(A)
    res = orc.lup_det(A, arith=orc.ARITH_LITERAL)
    out["ref_fixture_all/A32"] = raw
    out["ref_fixture_all/ref_det_f32"] = det32
    out["ref_fixture_all/ref_factor_digest"] = orc.factor_digests(fac32)
    out["ref_fixture_all/logabs"] = res["logabs"]
    out["ref_fixture_all/phase"] = res["phase"]
    out["ref_fixture_all/parity"] = res["parity"]
    out["ref_fixture_all/piv"] = res["piv"]
    out["ref_fixture_all/logabs_dd"] = la_dd
    out["ref_fixture_all/phase_dd"] = ph_dd
    np.savez_compressed(HERE / "golden_lup.npz", **out)
    print("wrote", HERE / "golden_lup.npz", sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
