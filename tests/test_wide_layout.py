"""Index arithmetic of the tensor-core engine, checked on the CPU: every
operand element, every byte an MMA descriptor reads and every raw matrix lies
inside its shared-memory buffer, the accumulators fit the tensor memory, and a
second CTA cannot be resident. Mirrors csrc/umma.cuh (CoreOffset,
SmemDescriptor) and csrc/wide_engine.cuh (Layout)."""
import pytest

CHUNK = 64
SBO = CHUNK // 4 * 128  # bytes between 8-row core-matrix groups
LBO = 128               # bytes between core matrices adjacent in depth
SMEM_PER_SM = 228 * 1024
SMEM_PER_CTA = 227 * 1024


def core_offset(row, k):
    return (row // 8) * SBO + (k // 4) * LBO + (row % 8) * 16 + (k % 4) * 4


def layout(kp):
    x_bytes = 128 * CHUNK * 4
    y_bytes = kp * CHUNK * 4
    vectors_at = 2 * x_bytes + 2 * y_bytes
    raw_count = 6 if kp == 64 else 0
    raw_bytes = kp * kp * 4
    raw_at = vectors_at + 6 * 128 * 4
    used = raw_at + raw_count * raw_bytes
    return {
        "xh": 0, "xl": x_bytes, "yh": 2 * x_bytes, "yl": 2 * x_bytes + y_bytes,
        "x_bytes": x_bytes, "y_bytes": y_bytes, "vectors_at": vectors_at,
        "raw_at": raw_at, "raw_bytes": raw_bytes, "raw_count": raw_count,
        "smem": max(used, 116 * 1024), "tmem_columns": 512,
        "columns": (0, kp, 2 * kp),
    }


@pytest.mark.parametrize("kp", [64, 128])
def test_operand_and_descriptor_bounds(kp):
    L = layout(kp)
    # Staged elements: X rows < 128, Y rows < KP, depth < CHUNK.
    assert max(core_offset(r, d) for r in range(128) for d in range(CHUNK)) + 4 <= L["x_bytes"]
    assert max(core_offset(r, d) for r in range(kp) for d in range(CHUNK)) + 4 <= L["y_bytes"]
    # An MMA at depth step k reads two core matrices (start, start + LBO) of
    # every 8-row group: M = 128 rows for X, N = KP rows for Y.
    for rows, size in ((128, L["x_bytes"]), (kp, L["y_bytes"])):
        for k in range(CHUNK // 8):
            start = k * 2 * LBO
            last = start + LBO + (rows // 8 - 1) * SBO + 127
            assert last < size
    # Buffers do not overlap and the vectors and raw matrices fit.
    assert L["xl"] + L["x_bytes"] <= L["yh"] and L["yh"] + L["y_bytes"] <= L["yl"]
    assert L["yl"] + L["y_bytes"] == L["vectors_at"]
    assert L["raw_at"] + L["raw_count"] * L["raw_bytes"] <= L["smem"] <= SMEM_PER_CTA
    assert L["raw_at"] % 16 == 0 and L["raw_bytes"] % 16 == 0
    # One CTA per SM: a second would have to wait on the tensor-memory allocation.
    assert 2 * L["smem"] > SMEM_PER_SM
    # The three accumulators (product, left and right adjoint factors).
    assert L["columns"][-1] + kp <= L["tmem_columns"]


def test_instruction_descriptor_fields():
    def tf32_descriptor(m, n):
        return (1 << 4) | (2 << 7) | (2 << 10) | ((n >> 3) << 17) | ((m >> 4) << 24)

    for n in (64, 128):
        d = tf32_descriptor(128, n)
        assert (d >> 4) & 3 == 1           # FP32 accumulator
        assert (d >> 7) & 7 == 2 and (d >> 10) & 7 == 2  # TF32 A and B
        assert (d >> 15) & 3 == 0          # both K-major
        assert ((d >> 17) & 63) << 3 == n
        assert ((d >> 24) & 31) << 4 == 128


# BF16 tier: the same buffers hold one BF16 operand in 8-row x 8-value core
# matrices (csrc/wide_engine.cuh CoreOffset16); one kind::f16 MMA reads a
# depth of 16 (two core matrices), so depth step k starts 256 bytes further.
SBO16 = CHUNK // 8 * 128


def core_offset16(row, k):
    return (row // 8) * SBO16 + (k // 8) * LBO + (row % 8) * 16 + (k % 8) * 2


@pytest.mark.parametrize("kp", [64, 128])
def test_bf16_operand_and_descriptor_bounds(kp):
    L = layout(kp)
    for rows, size in ((128, L["x_bytes"]), (kp, L["y_bytes"])):
        offsets = [core_offset16(r, d) for r in range(rows) for d in range(CHUNK)]
        # Every element in its own two bytes, inside the operand's hi buffer.
        assert len(set(offsets)) == len(offsets)
        assert max(offsets) + 2 <= size
        for k in range(CHUNK // 16):
            start = k * 2 * LBO
            last = start + LBO + (rows // 8 - 1) * SBO16 + 127
            assert last < size
    # A quad of depths 4q..4q+3 is 8 contiguous, 8-byte-aligned bytes.
    for r in range(0, kp, 7):
        for q in range(CHUNK // 4):
            base = core_offset16(r, 4 * q)
            assert base % 8 == 0
            assert [core_offset16(r, 4 * q + i) for i in range(4)] == [base + 2 * i
                                                                     for i in range(4)]


def test_bf16_instruction_descriptor_fields():
    def bf16_descriptor(m, n):
        return (1 << 4) | (1 << 7) | (1 << 10) | ((n >> 3) << 17) | ((m >> 4) << 24)

    for n in (64, 128):
        d = bf16_descriptor(128, n)
        assert (d >> 4) & 3 == 1                          # FP32 accumulator
        assert (d >> 7) & 7 == 1 and (d >> 10) & 7 == 1   # BF16 A and B (same type)
        assert (d >> 15) & 3 == 0
        assert ((d >> 17) & 63) << 3 == n
        assert ((d >> 24) & 31) << 4 == 128
