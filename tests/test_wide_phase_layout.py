"""Index arithmetic of the tensor-core phase kernels, checked on the CPU.
Mirrors csrc/wide_phase.cuh: PhaseLayout (operand parts, the unstored rows
64..127 of X at K_P = 64, TMEM columns, resident CTAs), the per-thread slot
walks of the operand staging (QuadCursor) and of the coalesced epilogues
(TileWalk), the epilogue tile, and the shared-memory transpose of the
adjoint ratio (TransposeStaged)."""
import pytest

CHUNK = 64
SBO = CHUNK // 4 * 128
SBO16 = CHUNK // 8 * 128
SMEM_PER_SM = 228 * 1024


def core_offset(row, k):
    return (row // 8) * SBO + (k // 4) * 128 + (row % 8) * 16 + (k % 4) * 4


def core_offset16(row, k):
    return (row // 8) * SBO16 + (k // 8) * 128 + (row % 8) * 16 + (k % 8) * 2


def layout(kp):
    threads = 128 if kp == 64 else 256
    part = kp * CHUNK * 4
    vectors_at = 4 * part
    used = vectors_at + 6 * 128 * 4
    columns = 128 if kp == 64 else 512
    per_sm = 512 // columns
    floor = SMEM_PER_SM // (per_sm + 1)
    smem = max(used, floor)
    resident = min(SMEM_PER_SM // (smem + 2048), per_sm)
    return dict(threads=threads, part=part, xh=0, xl=part, yh=2 * part, yl=3 * part,
                vectors_at=vectors_at, smem=smem, columns=columns, resident=resident)


@pytest.mark.parametrize("kp", [64, 128])
def test_layout_resources(kp):
    L = layout(kp)
    assert L["smem"] <= 227 * 1024
    # Forward split accumulators and the reverse's two products fit the columns.
    assert (kp // CHUNK + 1) * kp <= L["columns"] and 2 * kp <= L["columns"]
    # The resident CTAs never ask for more TMEM than the SM has.
    assert L["resident"] * L["columns"] <= 512
    assert L["resident"] == (3 if kp == 64 else 1)


@pytest.mark.parametrize("kp", [64, 128])
def test_mma_reads_stay_in_the_operand_buffers(kp):
    L = layout(kp)
    # An M = 128 X descriptor reads 128 rows from xh and from xl; an N = KP Y
    # descriptor reads KP rows from yh and yl (TF32: SBO 2048; BF16: 1024).
    for base in (L["xh"], L["xl"]):
        assert base + core_offset(127, CHUNK - 1) + 4 <= L["vectors_at"]
        assert base + core_offset16(127, CHUNK - 1) + 2 <= L["vectors_at"]
    for base in (L["yh"], L["yl"]):
        assert base + core_offset(kp - 1, CHUNK - 1) + 4 <= L["vectors_at"]
    # Staged (written) elements of X: rows < KP only, inside their own part.
    assert core_offset(kp - 1, CHUNK - 1) + 4 <= L["part"]
    # At KP = 64 the rows 64..127 that the X descriptors read alias the next
    # part: lanes nobody reads.
    if kp == 64:
        assert core_offset(64, 0) == L["part"]


def quad_cursor(K, depth, threads, tid, columns):
    """The slots thread `tid` visits, as (row, quad) or None for padding."""
    quads, quad_groups = depth // 4, (depth // 4 + 3) // 4
    if columns:
        major, minor = tid // K, tid % K
        step_major, step_minor, limit = threads // K, threads % K, K
        more = lambda: major < quads  # noqa: E731
    else:
        g, t = tid >> 5, tid & 31
        major, minor = g // quad_groups, g % quad_groups
        step_major = (threads // 32) // quad_groups
        step_minor = (threads // 32) % quad_groups
        limit = quad_groups
        more = lambda: major * 8 < K  # noqa: E731
    out = []
    while more():
        if columns:
            r, q = minor, major
        else:
            r, q = major * 8 + (t & 7), minor * 4 + (t >> 3)
        out.append((r, q) if r < K and q < quads else None)
        major += step_major
        minor += step_minor
        if minor >= limit:
            minor -= limit
            major += 1
    return out


@pytest.mark.parametrize("kp,threads", [(64, 128), (128, 256)])
@pytest.mark.parametrize("columns", [False, True])
def test_staging_walk_covers_every_quad_once(kp, threads, columns):
    for K in range(kp - 60, kp + 1, 4):  # K % 4 == 0 (the quad path)
        if K <= 32:
            continue
        for d0 in range(0, kp, CHUNK):
            depth = min(K - d0, CHUNK)
            seen = []
            for tid in range(threads):
                seen += [s for s in quad_cursor(K, depth, threads, tid, columns) if s]
            assert sorted(seen) == [(r, q) for r in range(K) for q in range(depth // 4)]


def tile_walk(K, threads, tid):
    quads = K // 4
    row, column = tid // quads, 4 * (tid % quads)
    step_rows, step_quads = threads // quads, threads % quads
    out = []
    while row < K:
        out.append((row, column))
        row += step_rows
        column += 4 * step_quads
        if column >= 4 * quads:
            column -= 4 * quads
            row += 1
    return out


@pytest.mark.parametrize("kp,threads", [(64, 128), (128, 256)])
def test_epilogue_walk_and_tile(kp, threads):
    L = layout(kp)
    for K in range(36, kp + 1, 4):
        seen = sorted(x for tid in range(threads) for x in tile_walk(K, threads, tid))
        assert seen == [(r, 4 * q) for r in range(K) for q in range(K // 4)]
        # The K x (K + 4) tile fits the idle operand buffers, and rows start
        # on 16-byte boundaries.
        stride = K + 4
        assert K * stride * 4 <= L["vectors_at"]
        assert (stride * 4) % 16 == 0
        # A thread's columns: [c0, c0 + KP / halves), every 32 columns a TMEM load.
        halves = threads // 128
        assert (kp // halves) % 32 == 0


def test_ratio_transpose_reads_one_core_matrix_row_set_per_step():
    # A warp moves an 8 x 4 block of X: lane -> (d, n) = (lane // 4, lane % 4);
    # the 32 reads fall in 32 distinct banks, the writes in two per bank.
    reads = {(core_offset(lane // 4, lane % 4) // 4) % 32 for lane in range(32)}
    assert len(reads) == 32
    writes = [(core_offset(lane % 4, lane // 4) // 4) % 32 for lane in range(32)]
    assert max(writes.count(b) for b in set(writes)) == 2
