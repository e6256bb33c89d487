"""Reader of the reference's DMHIST2 contact-history checkpoint
(src/cuda_backend_cuda.cu:545-656): magic "DMHIST2\\0", u32 version 2, u32
endian marker 0x01020304, u32 owners, u32 components, u32 slot counts
[64, 16, 64], u32 topology record size (40), u32 owner record size (188);
then per component (i32 id, i32 owner id, f64 radius, f64 body offset xyz),
per owner (i32 id, 23 f64 leapfrog state), then particle / wall / body keys
(u64) and values (9 f64 per slot)."""
import numpy as np


def read(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"DMHIST2\x00"
    head = np.frombuffer(raw, dtype="<u4", count=9, offset=8)
    version, endian, owners, comps, ps, ws, bs, topo, ownrec = (int(x) for x in head)
    off = 8 + 36
    trec = np.dtype([("id", "<i4"), ("owner", "<i4"), ("geo", "<f8", 4)])
    topo_arr = np.frombuffer(raw, dtype=trec, count=comps, offset=off)
    off += comps * trec.itemsize
    orec = np.dtype([("id", "<i4"), ("state", "<f8", 23)])
    own = np.frombuffer(raw, dtype=orec, count=owners, offset=off)
    off += owners * orec.itemsize
    keys, vals = [], []
    for slots in (ps, ws, bs):
        keys.append(np.frombuffer(raw, dtype="<u8", count=comps * slots, offset=off).reshape(comps, slots))
        off += comps * slots * 8
    for slots in (ps, ws, bs):
        vals.append(np.frombuffer(raw, dtype="<f8", count=comps * slots * 9, offset=off).reshape(comps, slots, 9))
        off += comps * slots * 72
    assert off == len(raw)
    return dict(version=version, endian=endian, owners=owners, comps=comps, slots=(ps, ws, bs), topo_size=topo,
                owner_size=ownrec, topology=topo_arr, owner_state=own, keys=keys, values=vals)
