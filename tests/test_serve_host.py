"""Host logic of the serving loop (admission, LRU offload, preemption,
latency accounting) with stand-in objects on CPU."""
import time

from supernormal_gb300.serve import Request, Server, poisson_trace


class FakeTrainer:
    B, P = 4, 9


class FakeObject:
    def __init__(self, nbytes, log):
        self._n, self.log, self.resident, self.last_used, self.tr = nbytes, log, True, 0.0, FakeTrainer()

    def nbytes(self):
        return self._n

    def offload(self):
        self.resident = False
        self.log.append(("off", id(self)))

    def onload(self):
        self.resident = True
        self.log.append(("on", id(self)))

    def train_iterations(self, n, graphs):
        time.sleep(0.002 * n)
        self.log.append(("train", id(self), n, graphs))

    def render(self, pose_seed):
        time.sleep(0.004)

        class Img:
            shape = (6, 6, 3)
        return Img()

    def query(self, res):
        time.sleep(0.003)


def test_admission_keeps_the_budget_and_evicts_least_recently_used():
    log = []
    objs = [FakeObject(100, log) for _ in range(4)]
    srv = Server(objs, 250, sync=lambda: None)
    srv.fit_budget()
    assert [o.resident for o in objs] == [True, True, False, False]
    objs[0].last_used, objs[1].last_used = 1.0, 2.0
    srv.admit(objs[2], 3.0)
    assert objs[2].resident and not objs[0].resident and objs[1].resident   # object 0 was the LRU
    assert srv.resident_bytes() <= 250
    srv.admit(objs[3], 4.0)
    assert objs[3].resident and not objs[1].resident and srv.resident_bytes() <= 250


def test_served_policy_preempts_reconstruction_for_short_requests():
    log = []
    objs = [FakeObject(10, log) for _ in range(2)]
    trace = [Request(0, "recon", 0, 0.0, 40), Request(1, "query", 1, 0.01), Request(2, "render", 1, 0.02)]
    res = Server(objs, 100, slice_iters=5, sync=lambda: None).run(trace, "served")
    assert res["requests"] == 3
    assert res["by_kind"]["query"]["p50_ms"] < res["by_kind"]["recon"]["p50_ms"]
    trains = [e for e in log if e[0] == "train"]
    assert len(trains) == 8 and all(e[2] == 5 and e[3] for e in trains)   # 40 iterations in slices of 5, graphs
    # the query ran before the reconstruction block finished
    assert res["by_kind"]["query"]["p99_ms"] < 1e3 * 0.002 * 40
    log.clear()
    res = Server(objs, 100, sync=lambda: None).run(trace, "plain")
    trains = [e for e in log if e[0] == "train"]
    assert len(trains) == 1 and trains[0][2] == 40 and not trains[0][3]   # one eager block
    assert res["by_kind"]["query"]["p50_ms"] >= 1e3 * 0.002 * 40 - 20     # waited behind the block


def test_poisson_trace_is_seeded_and_ordered():
    a = poisson_trace(5, 3.0, 10.0, seed=3)
    b = poisson_trace(5, 3.0, 10.0, seed=3)
    assert [(r.kind, r.obj, r.arrival) for r in a] == [(r.kind, r.obj, r.arrival) for r in b]
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    assert {r.kind for r in a} <= {"recon", "render", "query"} and all(0 <= r.obj < 5 for r in a)
