"""BlockId (core/block_id.rs:19-418): the 64-bit node id shared by the host API and the device.

Bit layout: 63 leaf flag | 62-55 child types | 54-47 child mask | 46-32 generation | 31-0 index.
EMPTY = 0 is a branch with mask 0 at index 0; INVALID = all ones.
"""

LEAF_SHIFT = 63
TYPES_SHIFT = 55
MASK_SHIFT = 47
GENERATION_SHIFT = 32
GENERATION_MASK = 0x7FFF
INDEX_MASK = 0xFFFFFFFF

INVALID = 0xFFFFFFFFFFFFFFFF
EMPTY = 0
MAX_INDEX = 0xFFFFFFFF
MAX_GENERATION = 0x7FFE


class BlockIdPanic(AssertionError):
    """Raised where BlockId asserts (block_id.rs:219, 273-276, 294-297, 316-321)."""


def new_extended(index, generation, types, mask, is_leaf):
    """block_id.rs:216-226."""
    if generation > MAX_GENERATION:
        raise BlockIdPanic("Generation overflow")
    return ((int(is_leaf) << LEAF_SHIFT) | ((types & 0xFF) << TYPES_SHIFT) | ((mask & 0xFF) << MASK_SHIFT)
            | ((generation & GENERATION_MASK) << GENERATION_SHIFT) | (index & INDEX_MASK))


def new_leaf(index, generation):
    return new_extended(index, generation, 0, 0, True)


def new_branch(index, generation, types, mask):
    return new_extended(index, generation, types, mask, False)


def index(raw):
    return raw & INDEX_MASK


def generation(raw):
    return (raw >> GENERATION_SHIFT) & GENERATION_MASK


def is_leaf(raw):
    return (raw >> LEAF_SHIFT) == 1


def is_branch(raw):
    return (raw >> LEAF_SHIFT) == 0


def is_empty(raw):
    return raw == EMPTY


def is_invalid(raw):
    return raw == INVALID


def is_valid(raw):
    return raw != INVALID


def types(raw):
    if not is_branch(raw):
        raise BlockIdPanic("Cannot get types from a leaf node")
    return (raw >> TYPES_SHIFT) & 0xFF


def mask(raw):
    if not is_branch(raw):
        raise BlockIdPanic("Cannot get mask from a leaf node")
    return (raw >> MASK_SHIFT) & 0xFF


def has_child(raw, child_index):
    if not is_branch(raw):
        raise BlockIdPanic("Cannot check child on a leaf node")
    if not 0 <= child_index < 8:
        raise BlockIdPanic("Child index out of bounds (0-7)")
    return (mask(raw) >> child_index) & 1 == 1


def describe(raw):
    """Display/Debug text (block_id.rs:420-470)."""
    if is_invalid(raw):
        return "Id(INVALID)"
    if is_empty(raw):
        return "Id(EMPTY)"
    if is_leaf(raw):
        return "Id(L, i: %08X, g: %04X)" % (index(raw), generation(raw))
    return "Id(B, i: %08X, g: %04X, m: %02X, t: %02X)" % (index(raw), generation(raw), mask(raw), types(raw))
