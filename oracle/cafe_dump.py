"""Reader for the per-step CA state records written by the test-only state
dumpers (oracle/ref_driver.cpp for the reference itself, and the oracle
restatement's own dump routine).

Record layout (little-endian):
  int32 magic 0x43414645, tag (0 initial, 1 after a step, 2 final CleanLayer),
  tInd, nGrain, ncell, isp, indlayer, inewlayerflg, inewscanflg; float64 time;
  int32 gID[ncell]; int32 vState[ncell]; float64 extents[ncell];
  float64 centroidOct[3*ncell]; float64 TempCurr[ncell]; int32 BuildjID[ncell];
  float64 cTheta[4*nGrain].
Test infrastructure only.
"""
import numpy as np

MAGIC = 0x43414645


def read_dump(path):
    data = open(path, "rb").read()
    off = 0
    recs = []
    while off < len(data):
        hdr = np.frombuffer(data, dtype="<i4", count=9, offset=off)
        if hdr[0] != MAGIC:
            raise ValueError("bad magic at offset %d" % off)
        tag, tind, ngrain, ncell, isp, indlayer, newlayer, newscan = [int(x) for x in hdr[1:]]
        off += 36
        time = float(np.frombuffer(data, dtype="<f8", count=1, offset=off)[0])
        off += 8
        r = dict(tag=tag, tInd=tind, nGrain=ngrain, ncell=ncell, isp=isp, indlayer=indlayer,
                 inewlayerflg=newlayer, inewscanflg=newscan, time=time)
        for name, dt, cnt in (("gID", "<i4", ncell), ("vState", "<i4", ncell),
                              ("extents", "<f8", ncell), ("centroid", "<f8", 3 * ncell),
                              ("temp", "<f8", ncell), ("buildj", "<i4", ncell),
                              ("cTheta", "<f8", 4 * ngrain)):
            arr = np.frombuffer(data, dtype=dt, count=cnt, offset=off)
            off += arr.nbytes
            r[name] = arr
        recs.append(r)
    return recs
