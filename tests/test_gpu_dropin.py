"""Native callers of the engine on the GPU, checked against the reference's files.

tests/native/dropin_loop.cpp runs the time loop over the drop-in classes of
include/amcafe/ (Grid, Partition, BasePlate, Utilities, TempField, VoxelsCA)
in the order main1.C calls them; tests/native/capi_loop.c runs it from C over
include/cafe_gpu.h. Both are compiled here against libcafe_gpu.so and write
the datasets of WriteToHDF1 at every output point. Every file the reference
wrote at those points (SHA-256 in tests/golden/output_digests.npz, made by
the reference's own sources, tests/golden/make_golden.py) must be
byte-identical.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def drivers(tmp_path_factory):
    from amcafe_gb300 import _native

    d = tmp_path_factory.mktemp("drivers")
    lib = os.path.dirname(_native.LIB_PATH)
    link = ["-L" + lib, "-lcafe_gpu", "-Wl,-rpath," + lib]
    inc = ["-I" + os.path.join(ROOT, "include", "amcafe"), "-I" + os.path.join(ROOT, "include")]
    cxx = str(d / "dropin_loop")
    cc = str(d / "capi_loop")
    subprocess.run(["g++", "-std=c++11", "-O2"] + inc + [os.path.join(HERE, "native", "dropin_loop.cpp"), "-o", cxx]
                   + link, check=True)
    subprocess.run(["gcc", "-std=c99", "-O2"] + inc + [os.path.join(HERE, "native", "capi_loop.c"), "-o", cc] + link,
                   check=True)
    return {"dropin": cxx, "capi": cc}


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


@pytest.mark.parametrize("driver", ["dropin", "capi"])
@pytest.mark.parametrize("name", ["layers_out_nl0", "layers_out_nl1", "track_nuc"])
def test_native_driver_output_matches_reference(drivers, driver, name, tmp_path):
    d = np.load(os.path.join(HERE, "golden", "output_digests.npz"))
    every = int(d[name + "/every"])
    r = subprocess.run([drivers[driver], os.path.join(HERE, "golden", "decks", name + ".in"), str(tmp_path)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    keys = [k.split("/", 1)[1] for k in d.files if k.startswith(name + "/") and not k.endswith("/every")]
    assert keys
    written = {f.split(".h5.")[0] for f in os.listdir(tmp_path) if ".h5." in f}
    want = {k.split(".h5.")[0] for k in keys}
    if every == 1:
        assert written == want, (sorted(written ^ want))[:10]
    else:
        assert want <= written
    for k in keys:
        path = tmp_path / k
        assert path.exists(), k
        assert _sha(path) == str(d[name + "/" + k]), "%s (%s driver): %s differs from the reference's file" % (
            name, driver, k)
