"""Reading the model payload written by vx_serialize_model (VoxModel::serialize,
world/voxmodel.rs:177-282, and serialize_chunk, world/voxchunk.rs:382-405) back on the host.

`decode` returns the stream as tables; `canonical` maps every chunk's root to a nested tuple that is
independent of the slot-index numbering, so two serialisations of the same model made by
implementations with different allocation orders compare equal. deserialize's reading order is the
reference's (voxmodel.rs:284-408): leaf count and leaves, branch count and branches (mask, one id per
set mask bit, LOD value), chunk count and chunk records.
"""


def _varint(b, p):
    v = s = 0
    while True:
        c = b[p]
        p += 1
        v |= (c & 0x7F) << s
        s += 7
        if c < 0x80:
            return v, p


def decode(b, voxel_bytes):
    """(leaves {id: value}, branches {id: (mask, [child ids], lod)}, chunks [((x, y, z), root id)])."""
    b = bytes(b)
    p = 0

    def u32(q):
        return int.from_bytes(b[q:q + 4], "big"), q + 4

    n, p = u32(p)
    leaves = {}
    for _ in range(n):
        i, p = _varint(b, p)
        leaves[i] = int.from_bytes(b[p:p + voxel_bytes], "big")
        p += voxel_bytes
    n, p = u32(p)
    branches = {}
    for _ in range(n):
        i, p = _varint(b, p)
        m = b[p]
        p += 1
        ch = []
        for k in range(8):
            if (m >> k) & 1:
                c, p = _varint(b, p)
                ch.append(c)
        lod = int.from_bytes(b[p:p + voxel_bytes], "big")
        p += voxel_bytes
        branches[i] = (m, ch, lod)
    n, p = u32(p)
    chunks = []
    for _ in range(n):
        if b[p:p + 12] != b"VoxTreeChunk":
            raise ValueError("chunk record without its VoxTreeChunk magic at byte %d" % p)
        p += 12
        pos = tuple(int.from_bytes(b[p + 4 * a:p + 4 * a + 4], "big", signed=True) for a in range(3))
        p += 12
        r, p = _varint(b, p)
        chunks.append((pos, r))
    if p != len(b):
        raise ValueError("%d trailing bytes" % (len(b) - p))
    return leaves, branches, chunks


def canonical(leaves, branches, chunks):
    """([(position, nested form of the root)], leaf count, branch count); forms are ('E',) for EMPTY,
    ('L', value) and ('B', mask, lod, child forms)."""
    memo = {}

    def form(i):
        if i == 0:
            return ("E",)
        f = memo.get(i)
        if f is not None:
            return f
        if i in leaves:
            f = ("L", leaves[i])
        else:
            m, ch, lod = branches[i]
            f = ("B", m, lod, tuple(form(c) for c in ch))
        memo[i] = f
        return f

    return [(pos, form(r)) for pos, r in chunks], len(leaves), len(branches)
