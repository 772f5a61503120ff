"""CPU checks of the index arithmetic the kernels use (no GPU): the node kernel's
multiply-shift division by GX, its 32-bit element-force offsets and the byte ranges the
persistent element kernel copies, restated here with 64-bit integers and checked
exhaustively at the benchmark mesh sizes and at edge sizes. A kernel given an index these
checks reject would read or write outside its buffer."""
import numpy as np
import pytest

# elements per axis: the five benchmark meshes, the test meshes and edge cases (one element,
# odd sizes, the largest mesh whose 3 N stays below 2^32)
MESHES = [(22, 22, 10), (96, 96, 40), (64, 64, 32), (48, 48, 24), (6, 5, 4), (10, 9, 6), (1, 1, 1), (2, 3, 5),
          (7, 1, 13), (255, 2, 3)]


def magic(GX):
    """The node kernel's constants for t / GX (capi.cu, ses3d_gpu_create)."""
    l = 0
    while (1 << l) < GX:
        l += 1
    m = ((1 << 32) * ((1 << l) - GX)) // GX + 1
    return m & 0xFFFFFFFF, l - 1


def magic_div(t, GX):
    m, shift = magic(GX)
    t = t.astype(np.uint64)
    hi = (t * np.uint64(m)) >> np.uint64(32)          # __umulhi(t, m)
    return ((hi + ((t - hi) >> np.uint64(1))) >> np.uint64(shift)).astype(np.int64)


@pytest.mark.parametrize("mesh", MESHES)
def test_node_division_exact(mesh):
    ex, ey, _ = mesh
    GX, GY = 4 * ex + 1, 4 * ey + 1
    t = np.arange(GX * GY, dtype=np.int64)
    assert np.array_equal(magic_div(t, GX), t // GX)


def test_node_division_exact_all_widths():
    """Every GX = 4 ex + 1 up to 4097, for every t of a square layer."""
    for ex in range(1, 1025):
        GX = 4 * ex + 1
        t = np.arange(0, GX * GX, max(1, GX * GX // 200000), dtype=np.int64)
        t = np.concatenate([t, np.arange(max(0, GX * GX - 2 * GX), GX * GX, dtype=np.int64)])
        assert np.array_equal(magic_div(t, GX), t // GX), GX


def node_force_offsets(mesh, gz):
    """Offsets of the (up to 8) element forces one layer of global nodes gathers, computed
    as k_node does (q0 plus the x, y, z steps, 32-bit unsigned) and as the definition
    force_offset(i, j, k, in, jn, kn) = 375 (i + ex (j + ey k)) + in + 5 jn + 25 kn."""
    ex, ey, ez = mesh
    GX, GY = 4 * ex + 1, 4 * ey + 1
    t = np.arange(GX * GY, dtype=np.int64)
    gy, gx = t // GX, t % GX
    i0 = np.where(gx == 0, 0, (gx - 1) >> 2)
    i1 = np.minimum(gx >> 2, ex - 1)
    j0 = np.where(gy == 0, 0, (gy - 1) >> 2)
    j1 = np.minimum(gy >> 2, ey - 1)
    k0 = 0 if gz == 0 else (gz - 1) >> 2
    k1 = min(gz >> 2, ez - 1)
    sy, sz = ex * 375, ex * 375 * ey
    M = 1 << 32
    q0 = ((i0 * 371 + gx) + (j0 * (sy - 20) + 5 * gy) + (k0 * (sz - 100) + 25 * gz)) % M
    dx = ((i1 - i0) * 371) % M
    dy = ((j1 - j0) * (sy - 20)) % M
    dz = ((k1 - k0) * (sz - 100)) % M
    out = []
    for a, (ii, da) in enumerate(((i0, 0), (i1, dx))):
        for b, (jj, db) in enumerate(((j0, 0), (j1, dy))):
            for c, (kk, dc) in enumerate(((k0, 0), (k1, dz))):
                got = (q0 + da + db + dc) % M
                want = 375 * (ii + ex * (jj + ey * kk)) + (gx - 4 * ii) + 5 * (gy - 4 * jj) + 25 * (gz - 4 * kk)
                out.append((got, want, ii, jj, kk))
    return out


@pytest.mark.parametrize("mesh", MESHES)
def test_node_force_offsets_in_bounds(mesh):
    """Every offset k_node reads (plus the component strides 125 and 250) lies inside the
    event's 3 N floats and equals the element's own node."""
    ex, ey, ez = mesh
    N = 125 * ex * ey * ez
    assert 3 * N < (1 << 32)
    GZ = 4 * ez + 1
    layers = range(GZ) if GZ * (4 * ex + 1) * (4 * ey + 1) < 4_000_000 else sorted(
        {0, 1, 2, 3, 4, 5, GZ // 2, GZ // 2 + 1, GZ - 5, GZ - 4, GZ - 3, GZ - 2, GZ - 1})
    for gz in layers:
        for got, want, ii, jj, kk in node_force_offsets(mesh, gz):
            assert np.array_equal(got, want), (mesh, gz)
            assert (ii >= 0).all() and (ii < ex).all() and (jj >= 0).all() and (jj < ey).all() and 0 <= kk < ez
            assert got.min() >= 0 and got.max() + 250 < 3 * N


def test_element_copy_ranges_inside_block():
    """Byte ranges of one element's state block (36 fields x 125 floats = 18,000 B) the
    persistent element kernel copies: full state, elastic (fields 0-17), lean (fields 0-5,
    and 18-35 with attenuation); 16-byte aligned, inside the block, covering the fields read."""
    block = 36 * 125 * 4
    ranges = {"full": [(0, block)], "elastic": [(0, 9008)], "lean_elastic": [(0, 3008)],
              "lean": [(0, 3008), (8992, 9008)]}
    fields_read = {"full": range(36), "elastic": range(18), "lean_elastic": range(6),
                   "lean": list(range(6)) + list(range(18, 36))}
    for name, rs in ranges.items():
        for a, n in rs:
            assert a % 16 == 0 and n % 16 == 0 and a + n <= block, name
        for f in fields_read[name]:
            lo, hi = f * 500, f * 500 + 500
            assert any(a <= lo and hi <= a + n for a, n in rs), (name, f)
    mat = 6 * 128 * 4
    assert block % 16 == 0 and mat % 16 == 0


def test_element_shared_memory_layout():
    """Dynamic shared memory of the persistent element kernel (kernels.cu: TMA_SMEM,
    tma_smem): the stage of one item (state block and material), the velocity and pressure
    buffers, the GLL tables, the 1-D table entries and the mbarrier; correlation items add
    the staged epilogue operands (12 floats and up to 8 doubles per point), lean record and
    correlation items two displacement stages. Every staged copy lands inside its buffer at
    its natural alignment, and the resident CTAs each shape asks for fit the SM's 228 KB
    (1 KB of it reserved per CTA)."""
    TPE, VBUF = 128, 2
    stage = 36 * 125 * 4 + 6 * 128 * 4                       # ElemStage, 16-byte aligned
    ktab = ((25 * 3 + 25 + 25 * 3 + 5) * 4 + 15) // 16 * 16  # KTab rounded to 16 bytes
    lt_off = stage + (9 + 3 * VBUF) * TPE * 4 + ktab
    bar_off = lt_off + VBUF * 48 * 4
    smem = bar_off + 8
    assert bar_off % 8 == 0 and stage % 16 == 0
    cs_off = (smem + 15) // 16 * 16
    cs_bytes = 12 * 128 * 4 + 8 * 128 * 8
    # staged operand addresses: floats [12][TPE], then doubles [8][TPE], thread n < 125
    n = np.arange(125)
    f_addr = cs_off + 4 * (np.arange(12)[:, None] * TPE + n[None, :])
    d_addr = cs_off + 12 * TPE * 4 + 8 * (np.arange(8)[:, None] * TPE + n[None, :])
    assert (f_addr % 4 == 0).all() and (d_addr % 8 == 0).all()
    assert f_addr.max() + 4 <= cs_off + 12 * TPE * 4 and d_addr.max() + 8 <= cs_off + cs_bytes
    sizes = {}
    for mode in range(6):
        corr, lean_rec = mode in (2, 5), mode in (4, 5)
        u_off = cs_off + cs_bytes if corr else cs_off
        size = u_off + 2 * 3 * TPE * 4 if lean_rec else (cs_off + cs_bytes if corr else smem)
        if lean_rec:   # displacement stages [2][3][TPE] floats
            u_addr = u_off + 4 * (np.arange(6)[:, None] * TPE + n[None, :])
            assert u_off % 16 == 0 and u_addr.max() + 4 <= size
        sizes[mode] = size
    # resident CTAs per SM: full-state modes run shape 0 (5 CTAs), lean record and
    # correlation modes shape 1 (4 CTAs), plain lean iterations every shape (up to 6)
    per_sm = 228 * 1024
    for mode, ctas in ((0, 6), (1, 5), (2, 5), (3, 6), (4, 4), (5, 4)):
        assert ctas * (sizes[mode] + 1024) <= per_sm, (mode, sizes[mode])
    # 44,208 B is the dynamic shared memory ncu reports for a MODE 2 launch
    assert sizes[2] == 44208 and sizes[5] == 47280
