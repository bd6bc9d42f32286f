"""The CPU oracle against the reference itself.

tests/golden/*.npz were produced by the reference's own sources (oracle/_ref,
built from AMCAFE src/src-mpi with single-rank shims; tests/golden/
make_golden.py). The oracle restatement with glibc libm must reproduce every
dumped record: integer fields bit for bit (SHA-256), float fields to 1e-12
relative (bit-exact on the machine that made the fixtures).
The correctly-rounded-libm mode (the arithmetic the GPU uses) must reproduce
the integer fields too on these decks (on two of them only for their first
steps, see CR_LATE). The track_easm and layers_easm decks run the EASM
temperature (TempField::EASM, Utilities.C), which the reference reaches only
with the CAFE_REF_EASM switch of its driver (its parser cannot select it).
"""
import hashlib
import os

import numpy as np
import pytest

import cafe_oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = ["track_r0", "track_nuc", "layers_rot", "c0_small", "track_easm", "track_easm60", "odd_dims", "track_p0",
         "layers_easm"]


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _rel(a, b):
    a, b = float(a), float(b)
    return 0.0 if a == b else abs(a - b) / max(abs(b), 1e-300)


def _check(name, libm, tmp_path, check_floats, deck=None, fixture=None):
    g = np.load(os.path.join(HERE, "golden", (fixture or name) + ".npz"))
    nsteps, stride = int(g["nsteps"]), int(g["stride"])
    dump = str(tmp_path / (name + ".bin"))
    orc.run(deck or os.path.join(HERE, "golden", "decks", name + ".in"), dump, max_steps=nsteps, dump_stride=stride,
            libm=libm)
    recs = orc.read_dump(dump)
    assert len(recs) == len(g["index"]), "%s: %d records vs %d in the fixture" % (name, len(recs), len(g["index"]))
    for j, r in enumerate(recs):
        where = "%s record %d" % (name, int(g["index"][j]))
        for f in ("tag", "tInd", "nGrain", "isp", "indlayer", "inewlayerflg", "inewscanflg"):
            assert r[f] == int(g[f][j]), "%s: %s %s vs %s" % (where, f, r[f], g[f][j])
        for f in ("gID", "vState", "buildj"):
            assert _digest(r[f]) == str(g["sha_" + f][j]), "%s: %s differs from the reference" % (where, f)
        if check_floats:
            for f in ("extents", "centroid", "temp", "cTheta"):
                assert _rel(np.nansum(r[f]), g["sum_" + f][j]) <= 1e-12, "%s: sum of %s" % (where, f)
    last = recs[-1]
    for f in ("gID", "vState", "buildj"):
        assert np.array_equal(last[f], g["last_" + f]), name
    if check_floats:
        for f in ("extents", "centroid", "temp", "cTheta"):
            a, b = last[f], g["last_" + f]
            same = (a == b) | (np.isnan(a) & np.isnan(b))
            if not same.all():
                d = np.abs(a - b)[~same] / np.maximum(np.abs(b)[~same], 1e-300)
                assert d.max() <= 1e-12, "%s: %s rel diff %g" % (name, f, d.max())


@pytest.mark.parametrize("name", DECKS)
def test_oracle_glibc_reproduces_reference(name, tmp_path):
    _check(name, orc.LIBM_GLIBC, tmp_path, check_floats=True)


# odd_dims and layers_easm are not among these: with correctly rounded libm
# their extents differ from the reference's in the last bits after a few steps
# (glibc rounds some capture-geometry or EASM value differently) and a capture
# decision flips later (steps 32 and 108); test_correctly_rounded_libm_diverges_late
# records that.
CR_LATE = {"odd_dims": 11, "layers_easm": 22}  # leading records whose integers agree
CR_DECKS = [d for d in DECKS if d not in CR_LATE]


@pytest.mark.parametrize("name", CR_DECKS)
def test_oracle_correctly_rounded_libm_keeps_reference_integers(name, tmp_path):
    _check(name, orc.LIBM_CR, tmp_path, check_floats=False)


@pytest.mark.parametrize("name", sorted(CR_LATE))
def test_correctly_rounded_libm_diverges_late(name, tmp_path):
    """The limit of the parity anchor: correctly rounded math reproduces the
    reference's grain IDs and states on odd_dims.in for its first 31 steps
    (records 0-10 at stride 3) and on layers_easm.in for its first 105 steps
    (records 0-21 at stride 5; its EASM temperatures differ in the last bits
    from step 1 and its extents from step 9, within 2e-15 relative), and
    differs after a capture decision that glibc's rounding changes (steps 32
    and 108)."""
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    dump = str(tmp_path / "o.bin")
    orc.run(os.path.join(HERE, "golden", "decks", name + ".in"), dump, max_steps=int(g["nsteps"]),
            dump_stride=int(g["stride"]), libm=orc.LIBM_CR)
    recs = orc.read_dump(dump)
    for j in range(CR_LATE[name]):
        for f in ("gID", "vState"):
            assert _digest(recs[j][f]) == str(g["sha_" + f][j]), (j, f)
    assert any(_digest(r["gID"]) != str(d) for r, d in zip(recs, g["sha_gID"]))


@pytest.mark.parametrize("name", sorted(CR_LATE))
def test_oracle_correctly_rounded_reproduces_reference_with_routed_libm(name, tmp_path):
    """On the two decks where glibc's rounding changes a capture decision, the
    reference's own code linked with the engine's libm routing (correctly
    rounded inside UpdateVoxels and EASM, glibc elsewhere;
    oracle/ref_shims/cr_route.cpp) produced tests/golden/<deck>_crlibm.npz.
    The correctly rounded oracle reproduces every record of it, floats
    included, to the end of the run: the restatement and the reference differ
    in nothing but libm's last bits."""
    _check(name, orc.LIBM_CR, tmp_path, check_floats=True, fixture=name + "_crlibm")


@pytest.mark.parametrize("libm", [orc.LIBM_GLIBC, orc.LIBM_CR])
def test_oracle_output_matches_reference(libm, tmp_path):
    """SetBuild and the datasets of WriteToHDF1 (gID, vState, Build, float
    Temperature, the three IPF colour maps, angle-axis table) at the output
    points, byte for byte against the reference's own files."""
    d = np.load(os.path.join(HERE, "golden", "output_digests.npz"))
    decks = sorted({k.split("/")[0] for k in d.files})
    assert decks
    for name in decks:
        out = tmp_path / name
        out.mkdir()
        orc.set_output(str(out), int(d[name + "/every"]))
        try:
            orc.run(os.path.join(HERE, "golden", "decks", name + ".in"), "", libm=libm)
        finally:
            orc.set_output(None)
        keys = [k for k in d.files if k.startswith(name + "/") and not k.endswith("/every")]
        assert keys
        for k in keys:
            path = out / k.split("/", 1)[1]
            assert path.exists(), k
            assert hashlib.sha256(path.read_bytes()).hexdigest() == str(d[k]), k


def test_seed_one_is_the_reference(tmp_path):
    """The extension keyword "seed" with s = 1 leaves the reference's seeds."""
    deck = tmp_path / "track_nuc_s1.in"
    with open(os.path.join(HERE, "golden", "decks", "track_nuc.in")) as f:
        deck.write_text(f.read() + "seed 1\n")
    _check("track_nuc", orc.LIBM_GLIBC, tmp_path, check_floats=True, deck=str(deck))


@pytest.mark.parametrize("name,pattern", [("track_nuc", 3), ("layers_rot", 4)])
def test_scan_patterns_3_and_4_run_as_1_and_2(name, pattern, tmp_path):
    """TempField.C:34-50 orders the laser points of patterns 3 and 4 exactly as
    those of 1 and 2 (the per-layer X/Y alternation that its comments at
    TempField.C:59-67 describe is not implemented), so the reference's records
    of a deck are the same with pattern 1 or 3 (2 or 4). The reference built
    here was run on both variants when this test was written and reproduced the
    pattern-1 and pattern-2 fixtures; the oracle must too."""
    import re

    src = open(os.path.join(HERE, "golden", "decks", name + ".in")).read()
    src2 = re.sub(r"(?mi)^patternID\s+\d+", "patternID %d" % pattern, src)
    assert src2 != src
    deck = tmp_path / ("%s_p%d.in" % (name, pattern))
    deck.write_text(src2)
    _check(name, orc.LIBM_GLIBC, tmp_path, check_floats=True, deck=str(deck))
