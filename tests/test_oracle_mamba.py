"""The oracle's Mamba probe table (oracle_mamba_*) against an independent
NumPy reading of editor/optix/probe.cuh, on the CPU.

- hash (probe.cuh:168-187): cell coordinates in 11 bits each, shuffled with
  an arithmetic right shift of a signed value, then two masked left
  shifts -- restated here with Python integers;
- the top table (request_L2 / lookup_L2, probe.cuh:560-712) probes
  linearly: every occupied slot's cell hashes to a slot at or before it,
  with no empty slot between;
- a second-level table (request_L1, probe.cuh:522-558) tries the hash's
  slot and the next: each probe sits in one of its two slots, under the
  hash of its own position, inside its table's 10-unit cell;
- probes are allocated one 16x16 block at a time in block order;
- the result does not depend on the number of host threads."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle

R = 32767
W, H = 128, 96
F = np.float32


def to_i32(v):
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v & 0x80000000 else v


def np_hash(center, size, res, x, d=(0, 0, 0)):
    idx = []
    for k in range(3):
        cd = (F(x[k]) - F(center[k])) + F(size) / F(2.0)
        idx.append(int(np.trunc((cd / F(res)) + F(d[k]))))
    u = (idx[0] & 0x7FF) | ((idx[1] & 0x7FF) << 11) | ((idx[2] & 0x7FF) << 22)
    h = to_i32(u)
    h ^= (h >> 11) ^ (h >> 22)
    u = h & 0xFFFFFFFF
    u ^= (u << 7) & 0x9D2C5680
    u &= 0xFFFFFFFF
    u ^= (u << 15) & 0xEFC60000
    return u & 0xFFFFFFFF


def lut_header(luts, l):
    row = luts[l]
    ints = row.view(np.int32)
    return {"center": row[0:3], "size": row[3], "resolution": row[4], "level": ints[5], "counter": ints[6]}


def render(name="box4k", frames=4, threads=0, direct=True):
    g = pyoracle.GeneratedScene(name, 1)
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), g.sah_bvh(4))
    cam = kgr.camera_dict(kgr.camera(g.eye, g.target, g.fov, W / H))
    m = pyoracle.Mamba(W, H, max_probes=1 << 12, max_luts=8)
    first = None
    for f in range(frames):
        p = pyoracle.mamba_params(W, H, cam, time=0.5 * f, samples=f, threads=threads, direct_lighting=int(direct),
                                  temporal_reuse=int(direct), spatial_reuse=int(direct))
        m.frame(osc, p)
        if f == 0:
            first = {k: m.buffer(k) for k in ("counters", "probe_pos", "g_position", "g_index")}
    return m, first


@pytest.fixture(scope="module")
def box():
    m, first = render()
    yield m, first
    m.close()


def test_top_table_header_and_linear_probing(box):
    m, _ = box
    luts, refs, hashes, pos = m.buffer("luts"), m.buffer("refs"), m.buffer("hashes"), m.buffer("lut_positions")
    nprobes, nluts = m.buffer("counters").ravel()
    top = lut_header(luts, 0)
    assert list(top["center"]) == [0, 0, 0] and top["size"] == 250 and top["resolution"] == 10 and top["level"] == 2
    occupied = np.nonzero(refs[:R] != -1)[0]
    assert len(occupied) == nluts - 1 == top["counter"]
    for j in occupied:
        c = pos[j, :3]
        h = np_hash(top["center"], top["size"], top["resolution"], c)
        assert hashes[j] == h
        k = (int(j) - h) % R
        between = [(h + i) % R for i in range(k)]
        assert all(refs[b] != -1 for b in between)
        assert 1 <= refs[j] < nluts
        sub = lut_header(luts, refs[j])
        assert sub["level"] == 1 and sub["size"] == 10 and sub["resolution"] == F(10) / F(25)
        assert np.array_equal(sub["center"], c)


def test_probes_sit_in_their_hash_slots(box):
    m, _ = box
    luts, refs, hashes, pos = m.buffer("luts"), m.buffer("refs"), m.buffer("hashes"), m.buffer("lut_positions")
    probe_pos = m.buffer("probe_pos")
    nprobes, nluts = m.buffer("counters").ravel()
    assert nprobes > 10
    seen = np.zeros(nprobes, bool)
    for l in range(1, nluts):
        sub = lut_header(luts, l)
        region = refs[l * R:(l + 1) * R]
        slots = np.nonzero(region != -1)[0]
        assert len(slots) == sub["counter"]
        for s in slots:
            p = region[s]
            assert 0 <= p < nprobes and not seen[p]
            seen[p] = True
            x = probe_pos[p, :3]
            assert np.array_equal(pos[l * R + s, :3], x)
            h = np_hash(sub["center"], sub["size"], sub["resolution"], x)
            assert hashes[l * R + s] == h and s in (h % R, (h + 1) % R)
            half = F(sub["size"]) / F(2)
            assert np.all(x >= sub["center"] - half) and np.all(x <= sub["center"] + half)
    assert seen.all()


def test_first_frame_allocates_in_block_order(box):
    """Before the first frame nothing is covered, so every 16x16 block is a
    candidate at its centre pixel; the probes are those centres, in block
    order, less the blocks whose centre is a miss or whose cell's two
    slots were already taken."""
    _, first = box
    n = first["counters"].ravel()[0]
    gpos, gidx = first["g_position"], first["g_index"]
    centres = []
    for b in range((W // 16) * (H // 16)):
        x, y = (b % (W // 16)) * 16 + 8, (b // (W // 16)) * 16 + 8
        if gidx[y * W + x] != -1:
            centres.append(gpos[y * W + x, :3])
    centres = np.array(centres)
    k = 0
    for p in range(n):
        while k < len(centres) and not np.array_equal(centres[k], first["probe_pos"][p, :3]):
            k += 1
        assert k < len(centres), f"probe {p} is not a later block centre"
        k += 1


def test_thread_count_does_not_change_the_state():
    a, _ = render(frames=3, threads=1)
    b, _ = render(frames=3, threads=8)
    for k in pyoracle.MAMBA_BUFFERS:
        x, y = a.buffer(k), b.buffer(k)
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), k
    a.close()
    b.close()


def test_bins_count_the_splats(box):
    """Every splat adds one to its bin's count and its radiance in fixed
    point: the counts are at most two per secondary pixel per frame and the
    sums decode to non-negative radiance for these non-negative lights."""
    m, _ = box
    bin_n, bin_le = m.buffer("bin_n"), m.buffer("bin_le").view(np.int64)
    nprobes = m.buffer("counters").ravel()[0]
    nsec = (W // 4 + 1) * (H // 4 + 1)
    assert 0 < bin_n.sum() <= 2 * nsec * 4
    assert bin_n[nprobes * 25:].sum() == 0
    assert (bin_le >= 0).all()
    used = bin_n[:nprobes * 25] > 0
    radiance = bin_le[:nprobes * 25][used] * 2.0 ** -20
    assert np.isfinite(radiance).all() and radiance.max() > 0
