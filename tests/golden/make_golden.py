"""Generates tests/golden/*.npz from the reference itself.

Runs oracle/_ref/cafe_ref_dump (AMCAFE's own sources built with single-rank
shims; see oracle/Makefile) on each deck in tests/golden/decks and stores, per
dumped record, SHA-256 digests of the integer fields and sums of the float
fields, plus the complete arrays of the last record. Needs the reference
checkout (to build oracle/_ref); run from the repository root:
    make -C oracle ref && python tests/golden/make_golden.py [deck ...]
The *_crlibm.npz fixtures come from the same driver linked with the engine's
libm routing (oracle/_ref/cafe_ref_dump_cr).
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from cafe_dump import read_dump  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "cafe_ref_dump")
# the reference with its libm calls routed as the engine evaluates them
# (oracle/ref_shims/cr_route.cpp): correctly rounded in the capture geometry,
# orientation sampling and EASM, glibc elsewhere -> <deck>_crlibm.npz
REF_CR = os.path.join(ROOT, "oracle", "_ref", "cafe_ref_dump_cr")
# deck, max steps (-1 = whole run), keep every k-th record. Decks named
# *easm* run the EASM temperature (CAFE_REF_EASM=1: the reference's parser
# cannot select it from a deck).
DECKS = [("track_r0", -1, 1), ("track_nuc", -1, 1), ("layers_rot", -1, 5), ("c0_small", 160, 10),
         ("track_easm", -1, 1), ("track_easm60", -1, 1), ("odd_dims", -1, 3), ("track_p0", -1, 1),
         ("layers_easm", 260, 5)]


# decks whose grain IDs under glibc's libm differ from those under correctly
# rounded libm (a capture decision flips at steps 32 and 108)
CR_DECKS = [("odd_dims", -1, 3), ("layers_easm", 260, 5)]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def summarize(recs, stride):
    keep = [i for i in range(len(recs)) if i == 0 or i == len(recs) - 1 or i % stride == 0]
    out = {"index": np.array(keep)}
    for f in ("tag", "tInd", "nGrain", "isp", "indlayer", "inewlayerflg", "inewscanflg"):
        out[f] = np.array([recs[i][f] for i in keep])
    for f in ("gID", "vState", "buildj"):
        out["sha_" + f] = np.array([digest(recs[i][f]) for i in keep])
    for f in ("extents", "centroid", "temp", "cTheta"):
        out["sum_" + f] = np.array([np.nansum(recs[i][f]) for i in keep])
    last = recs[-1]
    for f in ("gID", "vState", "buildj", "extents", "centroid", "temp", "cTheta"):
        out["last_" + f] = last[f]
    return out


def main(only=(), cr=False):
    ref = REF_CR if cr else REF
    if not os.path.exists(ref):
        sys.exit("build the reference first: make -C oracle ref")
    for name, nsteps, stride in (CR_DECKS if cr else DECKS):
        if only and name not in only:
            continue
        deck = os.path.join(HERE, "decks", name + ".in")
        env = dict(os.environ, CAFE_REF_EASM="1" if "easm" in name else "0")
        with tempfile.TemporaryDirectory() as td:
            dump = os.path.join(td, "ref.bin")
            cmd = [ref, deck, dump] + ([str(nsteps)] if nsteps > 0 else [])
            subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, env=env)
            recs = read_dump(dump)
        data = summarize(recs, stride)
        data["nsteps"] = np.array(nsteps)
        data["stride"] = np.array(stride)
        data["nrec"] = np.array(len(recs))
        out = name + ("_crlibm" if cr else "") + ".npz"
        np.savez_compressed(os.path.join(HERE, out), **data)
        print(out, len(recs), "records")


# Output of VoxelsCA::WriteToHDF1 (through the ADIOS2 shim's raw files) on
# three decks: deck, every k-th output point (outint is 1 in these decks).
OUTPUT_DECKS = [("track_r0", 10), ("track_nuc", 10), ("layers_rot", 40), ("layers_out_nl0", 1),
                ("layers_out_nl1", 1)]


def output_digests():
    """SHA-256 of every dataset file the reference writes (dims and VoxelDX
    aside) -> tests/golden/output_digests.npz, keys '<deck>/<file>'."""
    out = {}
    for name, every in OUTPUT_DECKS:
        deck = os.path.join(HERE, "decks", name + ".in")
        with tempfile.TemporaryDirectory() as td:
            env = dict(os.environ, CAFE_REF_DUMP_DIR=td, CAFE_REF_OUT_EVERY=str(every))
            subprocess.run([REF, deck, os.path.join(td, "ref.bin")], check=True, env=env,
                           stdout=subprocess.DEVNULL)
            for f in sorted(os.listdir(td)):
                if not f.endswith(".bin") or f == "ref.bin" or ".dims." in f or ".VoxelDX." in f:
                    continue
                with open(os.path.join(td, f), "rb") as fh:
                    out[name + "/" + f] = np.array(hashlib.sha256(fh.read()).hexdigest())
        out[name + "/every"] = np.array(every)
    np.savez_compressed(os.path.join(HERE, "output_digests.npz"), **out)
    print("output digests:", len(out))


if __name__ == "__main__":
    # optional arguments: deck names to regenerate (default: all, the
    # routed-libm fixtures and the output digests)
    main(tuple(sys.argv[1:]))
    main(tuple(sys.argv[1:]), cr=True)
    if len(sys.argv) == 1:
        output_digests()
