"""CPU: the one-launch many-shape executor's work items (tcfftDescribeManyItems,
host logic only, no GPU).

A plain-precision tcfftPlanMany plan runs every transform in one launch of
fft_many_kernel over a device item table.  These tests check the table the
planner builds:
* listed 1D transforms (N <= 2048) come first, in groups covering the row list once;
* every other transform's pass A and pass B items each cover its tiles exactly once, and its
  elements: a pass moves the whole transform;
* a pass-B item carries the number of its transform's pass-A items (what it waits for) and
  comes after all of them, at least the lag (10 x the SM count) later unless it is in the
  tail emitted after the last pass A;
* shapes the executor does not run are refused (the plan then replays its per-shape graph).
"""
import numpy as np
import pytest

import tcfft_gb300 as tc

LIST, PASS_B, PASS_A = 0x100, 0x200, 0x400


def uneven_workload(seed=2):
    """The uneven-batch workload of the benchmark: 512 1D transforms of 2^8..2^16 and 64 2D
    transforms of 2^7..2^10 per axis, shuffled."""
    rng = np.random.default_rng(seed)
    shapes = [(1 << int(e),) for e in rng.integers(8, 17, size=512)]
    shapes += [(1 << int(a), 1 << int(b)) for a, b in rng.integers(7, 11, size=(64, 2))]
    return [shapes[i] for i in rng.permutation(len(shapes))]


def size(shape):
    return int(np.prod(shape))


def check_items(shapes, items, num_sms):
    listed_1d = sum(1 for s in shapes if len(s) == 1 and s[0] <= 2048)
    listed_elems = sum(size(s) for s in shapes if len(s) == 1 and s[0] <= 2048)
    # listed groups first, covering row-list entries 0 .. listed_1d - 1 in order
    nlisted = elems = 0
    pos = 0
    while pos < len(items) and items[pos][0] & LIST:
        kind, first, _, cnt, tiles, e = items[pos]
        assert first == nlisted and 1 <= cnt <= 32 and tiles == 1
        nlisted += cnt
        elems += e
        pos += 1
    assert nlisted == listed_1d and elems == listed_elems
    assert not any(it[0] & LIST for it in items[pos:]), "a listed group after the passes"
    # per transform: tiles of each pass covered exactly once
    a_items, b_items = {}, {}
    last_a_index = -1
    for idx, (kind, xf, tile, cnt, tiles, e) in enumerate(items[pos:], start=pos):
        assert tiles >= 1 and tile >= 0 and 0 <= xf < len(shapes) and e > 0
        assert not (kind & PASS_A and kind & PASS_B)
        if kind & PASS_B:
            b_items.setdefault(xf, []).append((idx, tile, tiles, e, cnt))
        else:
            assert kind & PASS_A, "an item of neither pass"
            a_items.setdefault(xf, []).append((idx, tile, tiles, e))
            last_a_index = idx
    for d in (a_items, b_items):
        for xf, its in d.items():
            spans = sorted((t, t + n) for _, t, n, *_ in its)
            assert spans[0][0] == 0 and all(spans[i][1] == spans[i + 1][0] for i in range(len(spans) - 1)), \
                "tiles of transform %d not covered exactly once" % xf
            assert sum(it[3] for it in its) == size(shapes[xf]), "a pass of transform %d misses elements" % xf
    tail = last_a_index + 1
    lag = 10 * num_sms
    for xf, its in b_items.items():
        na = len(a_items.get(xf, []))
        assert all(cnt == na for *_, cnt in its), "pass-B items wait for the wrong count"
        first_b = min(idx for idx, *_ in its)
        if na:
            last_a = max(idx for idx, *_ in a_items[xf])
            assert first_b > last_a
            assert first_b >= tail or first_b - (last_a + 1) >= lag, \
                "transform %d: pass B %d items after its pass A (lag %d)" % (xf, first_b - last_a - 1, lag)
    # transforms with a pass: 1D above 2048 and every 2D shape; each has both passes
    assert set(a_items) == {i for i, s in enumerate(shapes) if len(s) == 2 or s[0] > 2048} == set(b_items)
    return len(items)


def test_uneven_workload_item_table():
    shapes = uneven_workload()
    items = tc.describe_many_items(shapes, num_sms=152)
    # the count the GPU plan reports for this workload ("2672 work items")
    assert check_items(shapes, items, 152) == 2672


@pytest.mark.parametrize("seed", [3, 4, 5])
@pytest.mark.parametrize("num_sms", [8, 148, 152])
def test_random_workloads(seed, num_sms):
    """num_sms 8 (lag 80 items) puts most pass-B items between other transforms' pass-A items,
    so the lag rule is exercised; at 148-152 the lag exceeds the pass-A items of these
    workloads and every pass B follows the last pass A."""
    shapes = uneven_workload(seed)
    items = tc.describe_many_items(shapes, num_sms=num_sms)
    check_items(shapes, items, num_sms)
    # the SM count sets the lag only, not the items
    assert sorted(items) == sorted(tc.describe_many_items(shapes, num_sms=num_sms + 4))


def test_single_shapes():
    for shape in [(256,), (2048,), (4096,), (1 << 15,), (1 << 16,), (128, 128), (1024, 2048), (2048, 128)]:
        items = tc.describe_many_items([shape] * 3)
        check_items([shape] * 3, items, 152)


@pytest.mark.parametrize("shapes", [[(1 << 17,)], [(4096, 4096)], [(256,), (64, 64)], [(16,)]])
def test_unsupported_shapes_are_refused(shapes):
    with pytest.raises(tc.TcfftError) as e:
        tc.describe_many_items(shapes)
    assert e.value.status == 7


def test_invalid_arguments():
    with pytest.raises(tc.TcfftError) as e:
        tc.describe_many_items([(256,)], num_sms=0)
    assert e.value.status == 1
