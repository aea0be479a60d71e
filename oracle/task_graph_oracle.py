"""Oracle of the device task graph — TEST INFRASTRUCTURE ONLY.

A sequential CPU restatement of the reference's task-graph executor
(shader/task-graph), used by tests/ as the checker of librdn's task-graph
kernels. Pure Python; sized for the small graphs of the tests.

    task record states                      runtime/task_pool.rs:118-139
    spawn (pop the empty pool, write the record, push the active list)
                                            runtime/task_group.rs:410-436, task_pool.rs:160-190
    wake (skip the push of a GO_TO_SLEEP task)
                                            runtime/task_group.rs:438-453
    poll / cleanup of a finished child      runtime/task_group.rs:455-495
    poll finalisation                       runtime/task_group.rs:130-165
    execute: per round, per group in order: prepare_execution (commit the
      active / empty / removed bump counters, drain removed into empty),
      poll every active task, commit + compaction
                                            runtime/mod.rs:357-397, task_group.rs:175-278
    bump allocate / deallocate / commit / drain
                                            bump_allocator.rs:83-316
    compaction (keep NOT_FINISHED_WAKEN, GO_TO_SLEEP -> SLEEP)
                                            runtime/dispatch_compact.rs:44-116
    init (empty pool 1..size, fallback task 0)
                                            runtime/task_group.rs:351-397
    execution states                        runtime/mod.rs:262-325
    futures: BaseShaderFuture resolves on its first poll (future/mod.rs:62-80);
      .then(spawn) spawns when its upstream resolves and polls the child at
      once (then.rs:56-78, task.rs:70-100); .map applies on resolution (map.rs)

Pushes and pops inside one poll are applied in active-list order here; on the
GPU their order follows the atomics, so only order-free quantities (counts,
state histograms, invariants) are compared beyond the first dispatch. A full
list, or an empty pool with nothing left, rejects the access and raises an
error flag (the reference's bound check admits one access past the end,
bump_allocator.rs:254-258, 296-300).
"""

from __future__ import annotations

from dataclasses import dataclass, field

NOT_EXIST, WAKEN, GO_TO_SLEEP, SLEEP, FINISHED = 0, 1, 2, 3, 4
NO_PARENT = 0xFFFFFFFF
UNINIT, RESOLVED = 0xFFFFFFFE, 0xFFFFFFFF
ERR_NO_FREE_SLOT, ERR_ACTIVE_FULL, ERR_REMOVED_FULL = 0x1, 0x2, 0x4


@dataclass
class _Bump:
    """A committed list plus the pushes / pops of the running dispatch."""

    items: list = field(default_factory=list)
    pending: list = field(default_factory=list)
    bump: int = 0


@dataclass
class _Group:
    spawns: list
    cap: int
    state: list
    parent_type: list
    parent_index: list
    locals: list
    active: _Bump
    removed: _Bump
    empty: _Bump


class OracleTaskGraph:
    """groups: list of (spawn_types, max_in_flight); a group's future is
    BaseShaderFuture, then one .then(spawn a task of each listed type with self
    as parent), then .map."""

    def __init__(self, groups, capacity: int):
        self.groups = []
        self.error = 0
        for spawns, mif in groups:
            cap = mif * capacity
            g = _Group(list(spawns), cap, [NOT_EXIST] * (cap + 1), [NO_PARENT] * (cap + 1),
                       [NO_PARENT] * (cap + 1), [[0, UNINIT, UNINIT, UNINIT, UNINIT] for _ in range(cap + 1)],
                       _Bump(), _Bump(), _Bump(items=list(range(1, cap + 1))))
            g.state[0] = WAKEN  # the fallback task
            self.groups.append(g)

    # --- bump lists ---
    def _push(self, g: _Group, lst: _Bump, idx: int, err: int):
        b = lst.bump
        lst.bump += 1
        if b < g.cap - len(lst.items):
            lst.pending.append(idx)
        else:
            self.error |= err

    @staticmethod
    def _commit_alloc(g: _Group, lst: _Bump):
        lst.items.extend(lst.pending[: g.cap - len(lst.items)])
        lst.pending = []
        lst.bump = 0

    @staticmethod
    def _commit_dealloc(lst: _Bump):
        keep = max(0, len(lst.items) - lst.bump)
        del lst.items[keep:]
        lst.bump = 0

    # --- task operations ---
    def _spawn(self, gi: int, parent_type: int, parent_index: int) -> int:
        g = self.groups[gi]
        esize = len(g.empty.items)
        b = g.empty.bump
        g.empty.bump += 1
        if b >= esize:
            self.error |= ERR_NO_FREE_SLOT
            return UNINIT
        idx = g.empty.items[esize - b - 1]
        g.state[idx] = WAKEN
        g.parent_type[idx] = parent_type
        g.parent_index[idx] = parent_index
        g.locals[idx] = [0, UNINIT, UNINIT, UNINIT, UNINIT]
        self._push(g, g.active, idx, ERR_ACTIVE_FULL)
        return idx

    def _wake(self, gi: int, idx: int):
        g = self.groups[gi]
        in_active = g.state[idx] == GO_TO_SLEEP
        g.state[idx] = WAKEN
        if not in_active:
            self._push(g, g.active, idx, ERR_ACTIVE_FULL)

    def _cleanup(self, gi: int, idx: int):
        g = self.groups[gi]
        self._push(g, g.removed, idx, ERR_REMOVED_FULL)
        g.state[idx] = NOT_EXIST

    def _poll_chain(self, gi: int, idx: int) -> bool:
        g = self.groups[gi]
        L = g.locals[idx]
        r = L[0] == 0
        L[0] = 1
        for k, cg in enumerate(g.spawns):
            if r:
                L[1 + k] = self._spawn(cg, gi, idx)
            r = False
            h = L[1 + k]
            if h not in (UNINIT, RESOLVED) and self.groups[cg].state[h] == FINISHED:
                self._cleanup(cg, h)
                L[1 + k] = RESOLVED
                r = True
        return r

    def _finalize(self, gi: int, idx: int, resolved: bool):
        g = self.groups[gi]
        if not resolved:
            g.state[idx] = GO_TO_SLEEP
            return
        g.state[idx] = FINISHED
        if g.parent_index[idx] == NO_PARENT:
            self._cleanup(gi, idx)
        else:
            self._wake(g.parent_type[idx], g.parent_index[idx])

    # --- executor steps ---
    def _prepare(self, gi: int):
        g = self.groups[gi]
        self._commit_alloc(g, g.active)
        self._commit_dealloc(g.empty)
        self._commit_alloc(g, g.removed)
        room = g.cap - len(g.empty.items)
        g.empty.items.extend(g.removed.items[:room])
        g.removed.items = []

    def _compact(self, gi: int):
        g = self.groups[gi]
        self._commit_alloc(g, g.active)
        kept = []
        for idx in g.active.items:
            st = g.state[idx]
            if st == GO_TO_SLEEP:
                g.state[idx] = SLEEP
            if st == WAKEN:
                kept.append(idx)
        g.active.items = kept

    def dispatch_allocate_init_task(self, count: int, gi: int):
        g = self.groups[gi]
        self._prepare(gi)
        for _ in range(count):
            self._spawn(gi, NO_PARENT, NO_PARENT)
        self._commit_alloc(g, g.active)
        self._commit_dealloc(g.empty)

    def execute(self, rounds: int):
        for _ in range(rounds):
            for gi in range(len(self.groups)):
                self._prepare(gi)
                for idx in list(self.groups[gi].active.items):
                    self._finalize(gi, idx, self._poll_chain(gi, idx))
                self._compact(gi)

    def read_back_execution_states(self):
        for gi in range(len(self.groups)):
            self._prepare(gi)
            self._compact(gi)
        wake = [len(g.active.items) for g in self.groups]
        empty = [len(g.empty.items) for g in self.groups]
        sleep = [g.cap - e - w for g, e, w in zip(self.groups, empty, wake)]
        return wake, sleep, empty

    def debug_execution(self):
        self.read_back_execution_states()
        return [(list(g.active.items), list(g.empty.items), list(g.state)) for g in self.groups]
