"""Reader of MPIIO result files, restating the steps of the reference's
bin2vtu.py (main, bin2vtu.py:18-150; readHeader :190-205; readInString
:208-220): a '\\x01'-terminated banner, the uint64 header, point and cell field
names, float32 node coordinates, uint64 connectivity / offsets / types, then
datasets of uint64 iteration + float32 point and cell fields.  Test helper
only: it checks files the library writes."""
import numpy as np


class _Cursor:
    def __init__(self, raw):
        self.raw, self.pos = raw, 0

    def string(self):
        end = self.raw.index(b"\x01", self.pos)
        s = self.raw[self.pos:end].decode()
        self.pos = end + 1
        return s

    def array(self, dtype, n):
        a = np.frombuffer(self.raw, dtype=dtype, count=n, offset=self.pos)
        self.pos += a.nbytes
        return a


def read_result_file(path):
    """dict with banner, header counts, names, points (nn, 3), cells (nel, 8),
    offsets, types and datasets [(itr, point fields (npf, nn), cell fields
    (ncf, nel))]."""
    raw = open(path, "rb").read()
    c = _Cursor(raw)
    out = {"banner": c.string()}
    ndom = int(c.array("<u8", 1)[0])
    counts = c.array("<u8", 4 * ndom)
    npe = int(c.array("<u8", 1)[0])
    assert ndom == 1, "one domain"
    nn, nel, npf, ncf = (int(v) for v in counts)
    out.update(nDom=ndom, nPointsT=nn, nCellsT=nel, nPFields=npf, nCFields=ncf, nodesPerElement=npe)
    out["pointFieldNames"] = [x.strip() for x in c.string().split(",")]
    out["cellFieldNames"] = [x.strip() for x in c.string().split(",")]
    out["points"] = c.array("<f4", 3 * nn).reshape(nn, 3)
    out["cells"] = c.array("<u8", 8 * nel).reshape(nel, 8)
    out["offsets"] = c.array("<u8", nel)
    out["types"] = c.array("<u8", nel)
    ds = []
    while c.pos < len(raw):
        itr = int(c.array("<u8", 1)[0])
        pf = c.array("<f4", npf * nn).reshape(npf, nn)
        cf = c.array("<f4", ncf * nel).reshape(ncf, nel)
        ds.append((itr, pf, cf))
    out["datasets"] = ds
    return out


def point_fields_of(*vectors):
    """The float32 point-field block of DOF-interleaved nodal vectors: field
    3 v + c holds component c of vector v (MPIIO.cc:289-340)."""
    return np.concatenate([np.asarray(u, dtype=np.float64).reshape(-1, 3).T.astype(np.float32) for u in vectors])
