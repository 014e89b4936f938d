"""The lattice kernel's phase waits (levels.cu, lt_wait_phase and the item
loop of k_lattice) restated as interleaved workers under sequentially
consistent memory. Workers pop items in order; an item of phase k > 0 first
waits until phase k - 1 has counted all its items; a wait that runs out sets
the status, and a skipped item still counts. The invariant: an item runs
only when every item of the phase before it ran. With the host's fault
injection (the first phase counts one item more than exists) the waits of
the second phase run out. Reading the status after a full counter keeps the
invariant under every interleaving tried; the earlier order (the status only
while the counter is short) breaks it, which is the fault the kernel had.
CPU only."""
import random

import pytest


def simulate(ph_size, workers, wait_limit, seed, status_after_counter, fault):
    items = [ph for ph, size in enumerate(ph_size) for _ in range(size)]
    want = list(ph_size)
    if fault:
        want[0] += 1  # the first phase counts one item more than exists
    done = [0] * len(ph_size)
    ran = [0] * len(ph_size)
    mem = {"next": 0, "status": 0}
    violations = []

    def worker():
        while True:
            it = mem["next"]
            mem["next"] += 1
            yield
            if it >= len(items):
                return
            ph = items[it]
            run = True
            if ph > 0:
                run = False
                for _ in range(wait_limit):
                    full = done[ph - 1] >= want[ph - 1]
                    yield
                    if full:
                        run = mem["status"] == 0 if status_after_counter else True
                        break
                    if mem["status"] != 0:
                        break
                    yield
                else:
                    mem["status"] = 1
                yield
            if run:
                if ph > 0 and ran[ph - 1] != len([i for i in items if i == ph - 1]):
                    violations.append(it)
                ran[ph] += 1
            yield
            done[ph] += 1
            yield

    rng = random.Random(seed)
    live = [worker() for _ in range(workers)]
    while live:
        w = rng.choice(live)
        try:
            next(w)
        except StopIteration:
            live.remove(w)
    return violations, mem["status"], ran


PHASES = [3, 5, 2, 4, 3, 6, 2]


@pytest.mark.parametrize("workers", [2, 3, 5, 8])
def test_no_item_runs_after_a_wait_ran_out(workers):
    for seed in range(60):
        v, status, ran = simulate(PHASES, workers, 6, seed, True, fault=True)
        assert not v, (workers, seed, v)
        assert status == 1
        # the first phase has no wait and runs; nothing after it does
        assert ran == [PHASES[0]] + [0] * (len(PHASES) - 1), (workers, seed, ran)


@pytest.mark.parametrize("workers", [1, 2, 4, 8])
def test_without_fault_every_item_runs(workers):
    for seed in range(30):
        v, status, ran = simulate(PHASES, workers, 10 ** 6, seed, True, fault=False)
        assert not v and status == 0 and ran == PHASES, (workers, seed, ran)


def test_the_earlier_order_lets_later_phases_run_on_skipped_inputs():
    found = 0
    for workers in (3, 5, 8):
        for seed in range(60):
            v, _, _ = simulate(PHASES, workers, 6, seed, False, fault=True)
            found += bool(v)
    assert found > 0
