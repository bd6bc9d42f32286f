"""Output of the GPU engine (SetBuild + WriteToHDF1) against the reference's own files.

tests/golden/output_digests.npz holds the SHA-256 of every dataset file that
the reference (oracle/_ref, built from AMCAFE's sources) wrote at the output
points of its decks (tests/golden/make_golden.py). Here all five run through
the C ABI (two of them, layers_out_nl0/1, write every 20th step, and at each
layer change only when outnl is 0, main1.C:77-84): cafe_sim_step calls
SetBuild at each output point and writes the datasets there
(cafe_sim_set_output), and after the closing CleanLayer they are written
with cafe_sim_write_output. Every file must be
byte-identical to the reference's: gID, vState, Build, the float temperature,
the three IPF colour maps (computed on the device) and the angle-axis table.
"""
import hashlib
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = os.path.join(HERE, "golden", "decks")


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _run_deck(name, every, out):
    """The loop with the engine writing each output point itself
    (cafe_sim_set_output: before the step's AddLayer1, main1.C:79-88), then
    the closing CleanLayer and its write (main1.C:95-97) as "final"."""
    from amcafe_gb300 import Simulation

    sim = Simulation(os.path.join(DECKS, name + ".in"), device=0)
    sim.set_output(str(out / "out"))
    sim.InitializeVoxels()
    sim.begin()
    done = False
    while not done:
        done = sim.step()
    sim.CleanLayer()
    sim.WriteToHDF1(str(out / "final.h5"))
    written = sorted({f.split(".h5.")[0] for f in os.listdir(out) if ".h5." in f})
    return sim, written


@pytest.mark.parametrize("name", ["track_r0", "track_nuc", "layers_rot", "layers_out_nl0", "layers_out_nl1"])
def test_output_files_match_reference(name, tmp_path):
    d = np.load(os.path.join(HERE, "golden", "output_digests.npz"))
    every = int(d[name + "/every"])
    sim, written = _run_deck(name, every, tmp_path)
    keys = [k.split("/", 1)[1] for k in d.files if k.startswith(name + "/") and not k.endswith("/every")]
    assert keys
    # the same output points as the reference (which kept every k-th)
    want = sorted({k.split(".h5.")[0] for k in keys})
    if every == 1:
        assert want == written
    else:
        assert set(want) <= set(written)
    for k in keys:
        path = tmp_path / k
        assert path.exists(), k
        assert _sha(path) == str(d[name + "/" + k]), "%s: %s differs from the reference's file" % (name, k)
    # dims and VoxelDX, and the in-memory downloads against the files
    info = sim.info()
    fin = str(tmp_path / "final.h5.")
    assert np.fromfile(fin + "dims.bin", np.int32).tolist() == [info["nx"], info["ny"], info["nz"]]
    assert np.fromfile(fin + "VoxelDX.bin", np.float32)[0] == np.float32(info["dx"])
    assert np.array_equal(sim.build(), np.fromfile(fin + "Build.bin", np.int32))
    o = sim.output()
    for k in ("Temperature", "IPFz", "IPFx", "IPFy"):
        assert o[k].tobytes() == open(fin + k + ".bin", "rb").read(), k
    # the XDMF description names each per-cell file with its shape
    root = ET.parse(str(tmp_path / "final.h5.xdmf")).getroot()
    topo = root.find(".//Topology").get("Dimensions").split()
    assert [int(v) for v in topo] == [info["nz"] + 1, info["ny"] + 1, info["nx"] + 1]
    names = []
    for att in root.iter("Attribute"):
        item = att.find("DataItem")
        dims = [int(v) for v in item.get("Dimensions").split()]
        f = tmp_path / item.text
        assert f.exists(), item.text
        assert f.stat().st_size == 4 * int(np.prod(dims)), item.text
        names.append(att.get("Name"))
    assert names == ["gID", "vState", "Build", "Temperature", "IPFz", "IPFx", "IPFy"]
    sim.close()
