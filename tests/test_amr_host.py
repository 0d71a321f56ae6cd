"""The host-side plan of a regrid inside the same patch arena
(amr.in_place_slots, the bookkeeping of TwoLevel.set_blocks): every new slot
gets exactly one block, kept patches below the new count stay where they are,
kept patches above it move into free slots, new patches take the rest, and the
box copies read only slots that no copy writes."""
import numpy as np
import pytest

from axion_strings_adaptive_gb300 import _lib as L
from axion_strings_adaptive_gb300.amr import in_place_slots


def _old_slots(rng, n_old, n_new):
    """old_q for a new set of n_new blocks: a random subset of the n_old old
    patches is kept, at random positions of the new list; the rest are new."""
    old_q = np.full(n_new, -1, dtype=np.int64)
    if n_old == 0:
        return old_q
    n_keep = int(rng.integers(0, min(n_old, n_new) + 1))
    kept = rng.choice(n_old, size=n_keep, replace=False)
    old_q[rng.choice(n_new, size=n_keep, replace=False)] = kept
    return old_q


def _check(old_q, n_new):
    slot, sod, fresh = in_place_slots(old_q, n_new)
    assert sorted(slot.tolist()) == list(range(n_new))  # a permutation of the new slots
    for i, q in enumerate(old_q):
        s = slot[i]
        if 0 <= q < n_new:
            assert s == q and sod[s] == L.PATCH_KEEP  # stays in place
        elif q >= n_new:
            assert sod[s] == q  # moves down from above the new count
        else:
            assert sod[s] == -1  # newly refined: cleared, then interpolated
    assert sorted(fresh.tolist()) == sorted(slot[old_q < 0].tolist())
    copied = sod[(sod != L.PATCH_KEEP) & (sod >= 0)]
    assert np.all(copied >= n_new)  # sources lie past every destination
    return slot, sod


@pytest.mark.parametrize("seed", range(40))
def test_in_place_slot_plan_random(seed):
    rng = np.random.default_rng(seed)
    cap = int(rng.integers(1, 300))
    n_old, n_new = int(rng.integers(0, cap + 1)), int(rng.integers(1, cap + 1))
    _check(_old_slots(rng, n_old, n_new), n_new)


def test_in_place_slot_plan_cases():
    # nothing kept: new patches fill 0..n-1 in order
    slot, sod = _check(np.full(4, -1), 4)
    assert slot.tolist() == [0, 1, 2, 3] and sod.tolist() == [-1] * 4
    # everything kept in place
    slot, sod = _check(np.array([2, 0, 1]), 3)
    assert slot.tolist() == [2, 0, 1] and sod.tolist() == [L.PATCH_KEEP] * 3
    # a shrink: patches 5 and 4 move into the holes 1 and 3, in list order
    slot, sod = _check(np.array([0, 5, 2, 4]), 4)
    assert slot.tolist() == [0, 1, 2, 3] and sod.tolist() == [L.PATCH_KEEP, 5, L.PATCH_KEEP, 4]
    # movers take the first holes, new patches the ones after them
    slot, sod = _check(np.array([-1, 7, 1]), 3)
    assert slot.tolist() == [2, 0, 1] and sod.tolist() == [7, L.PATCH_KEEP, -1]
