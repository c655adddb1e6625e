"""Round selection of the serving loop, on the CPU with a stand-in batch."""
import numpy as np
import pytest

from pixelflow_gb300.geometry import Request
from pixelflow_gb300.config import Settings
from pixelflow_gb300.serve import Server, summarize


class FakeBatch:
    """Records every round; a step costs one time unit per million cells."""

    def __init__(self):
        self.slots, self.rounds, self.clock = {}, [], 0.0

    def memory(self):
        return (0, 1 << 60)

    def add_shapes(self, settings, shape, shapes, edge):
        slot = len(self.slots)
        self.slots[slot] = {"cells": int(np.prod(shape)), "done": 0}
        return slot

    def step_slots(self, slots, steps):
        self.rounds.append(list(zip(slots, steps)))
        for s, k in zip(slots, steps):
            self.slots[s]["done"] += k

    def last_ms(self):
        return 0.0

    def norms(self, slot):
        return (1.0, 0.0)

    def get_state(self, slot):
        return {"steps": self.slots[slot]["done"]}

    def remove(self, slot):
        pass

    def close(self):
        pass


def _requests():
    s = Settings()
    sizes = [(64, 64), (512, 512), (128, 128), (32, 32, 32), (256, 256), (96, 96, 96)]
    steps = [40, 100, 10, 60, 30, 20]
    return [Request(i, 0.0, len(sh), sh, s, [], st) for i, (sh, st) in enumerate(zip(sizes, steps))]


@pytest.mark.parametrize("policy", ["rr", "srpt", "srpt_fill"])
def test_every_request_gets_exactly_its_steps(policy, monkeypatch):
    import pixelflow_gb300.serve as S
    monkeypatch.setattr(S, "case_bytes", lambda *a, **k: 1)
    fb = FakeBatch()
    srv = Server(chunk=10, policy=policy, round_cells=300_000, batch=fb)
    res = srv.run(_requests(), realtime=False)
    assert [r.state["steps"] for r in res] == [q.steps for q in _requests()]
    if policy == "rr":
        assert len(fb.rounds[0]) == 6
    elif policy == "srpt_fill":
        # least remaining work first; each case the steps it runs alone in
        # round_ms; the round's cell-steps within the budget (one case at least)
        first = fb.rounds[0]
        work = {i: r.cells * r.steps for i, r in enumerate(_requests())}
        assert first[0][0] == min(work, key=work.get)
        for s, k in first:
            r = _requests()[s]
            assert 1 <= k <= min(r.steps, max(1, int(srv.round_ms / srv._step_ms(r.cells, r.dim))))
        assert sum(_requests()[s].cells * k for s, k in first[:-1]) < srv.round_work
    else:
        # the first round holds the least remaining work first, until 300k cells
        first = [s for s, _ in fb.rounds[0]]
        work = {i: r.cells * r.steps for i, r in enumerate(_requests())}
        assert first[0] == min(work, key=work.get)
        assert sum(_requests()[s].cells for s in first[:-1]) < 300_000


def test_srpt_finishes_short_requests_first(monkeypatch):
    """With a round's GPU time proportional to the cell-steps it runs, srpt
    completes the cheap requests earlier and lowers the mean completion time,
    for the same total work and the same completion time of the last request."""
    import pixelflow_gb300.serve as S
    monkeypatch.setattr(S, "case_bytes", lambda *a, **k: 1)
    reqs = _requests()
    finish, total = {}, {}
    for policy in ("rr", "srpt"):
        fb = FakeBatch()
        srv = Server(chunk=10, policy=policy, round_cells=50_000, batch=fb)
        srv.run(reqs, realtime=False)
        left = {i: r.steps for i, r in enumerate(reqs)}
        clock, finish[policy] = 0, {}
        for rnd in fb.rounds:
            clock += sum(reqs[s].cells * k for s, k in rnd)
            for s, k in rnd:
                left[s] -= k
                if left[s] == 0:
                    finish[policy][s] = clock
        total[policy] = clock
    assert total["rr"] == total["srpt"]
    assert max(finish["srpt"].values()) == max(finish["rr"].values())
    work = {i: r.cells * r.steps for i, r in enumerate(reqs)}
    cheapest = min(work, key=lambda i: (work[i], reqs[i].steps))
    assert finish["srpt"][cheapest] < finish["rr"][cheapest]
    assert np.mean(list(finish["srpt"].values())) < np.mean(list(finish["rr"].values()))


def test_srpt_fill_finishes_cheap_requests_in_fewer_rounds(monkeypatch):
    """With a round lasting as long as its slowest case (each case's steps x
    its modelled step time, at least the round's cell-steps at the GPU's
    rate), srpt_fill completes the cheap requests much earlier than srpt,
    which gives every case of a round the same chunk, and the last request
    no later than srpt does."""
    import pixelflow_gb300.serve as S
    monkeypatch.setattr(S, "case_bytes", lambda *a, **k: 1)
    s = Settings()
    sizes = [(192, 192), (288, 288), (1024, 1024), (192, 192, 192), (64, 64, 64), (320, 320), (160, 160, 160)]
    steps = [900, 350, 400, 500, 900, 750, 800]
    reqs = [Request(i, 0.0, len(sh), sh, s, [], st) for i, (sh, st) in enumerate(zip(sizes, steps))]
    finish = {}
    for policy in ("srpt", "srpt_fill"):
        fb = FakeBatch()
        srv = Server(chunk=25, policy=policy, round_cells=24_000_000, batch=fb)
        srv.run(reqs, realtime=False)
        left = {i: r.steps for i, r in enumerate(reqs)}
        clock, finish[policy] = 0.0, {}
        for rnd in fb.rounds:
            slowest = max(k * srv._step_ms(reqs[q].cells, reqs[q].dim) for q, k in rnd)
            clock += max(slowest, sum(reqs[q].cells * k for q, k in rnd) / 1.3e9 * 1e3)
            for q, k in rnd:
                left[q] -= k
                if left[q] == 0:
                    finish[policy][q] = clock
    cheap = sorted(range(len(reqs)), key=lambda i: reqs[i].cells * reqs[i].steps)[:3]
    for i in cheap:
        assert finish["srpt_fill"][i] < 0.5 * finish["srpt"][i]
    assert np.median(list(finish["srpt_fill"].values())) < np.median(list(finish["srpt"].values()))
    assert max(finish["srpt_fill"].values()) <= max(finish["srpt"].values())
