"""Proof serving with continuous batching.

This is the request loop of the reference's proof server
(proof-server/src/prover_backend.rs:88-107 enters proof execution per
request; transient-crypto/src/proofs.rs:196-230 selects the accelerator).
It is rebuilt around one GPU:

  * every circuit's proving key (fixed columns, cosets, permutation data)
    and the SRS bases of every size stay resident on the device, and are
    built once when the server starts;
  * `slots` worker threads each own an execution lane, which has its own
    CUDA stream, so the kernels of proofs in flight overlap on the device
    and their host steps overlap with other proofs' device work;
  * admission is continuous. A request starts as soon as a worker is free
    and its estimated device footprint fits in what is left of the HBM
    budget. The oldest waiting request that fits goes first, and nothing
    waits for a batch to fill;
  * each request's bytes depend only on the request (its witness and its
    prover-rng seed), never on what else is in flight.
"""
import collections
import threading
import time
from concurrent.futures import Future

import numpy as np

from . import api
from .kzg import CircuitTranscript
from .plonk import GpuBackend, create_proof, create_proofs
from .rng import ChaCha20Rng


def proof_footprint_bytes(circuit):
    """Device bytes one proof of this circuit holds at its peak: extended
    cosets of the advice, permutation and lookup columns and the numerator;
    Lagrange and coefficient forms; MSM scratch for the largest batch."""
    n = circuit.n
    ext = n * (1 << max(1, (circuit.cs_degree - 2).bit_length()))
    L, m, sets = circuit.lookups, circuit.m, circuit.permutation_sets
    ext_cols = m + sets + 3 * L + 2
    n_cols = 3 * (m + sets + 3 * L) + 12
    msm_scratch = n * max(m, 4) * 24 * 4
    return 32 * (ext * ext_cols + n * n_cols) + msm_scratch


class Request:
    __slots__ = ("circuit_id", "witness", "seed", "arrival", "start", "finish", "future", "bytes", "proof",
                 "params", "pk", "backend")

    def __init__(self, circuit_id, witness, seed, nbytes, params, pk, backend):
        self.circuit_id, self.witness, self.seed, self.bytes = circuit_id, witness, seed, nbytes
        self.params, self.pk, self.backend = params, pk, backend
        self.arrival = time.perf_counter()
        self.start = self.finish = None
        self.future = Future()
        self.proof = None


class KeyStore:
    """Proving keys by the SHA-256 of their key-file bytes (keyfile.py), built
    resident on first use and kept for the `capacity` most recently used
    keys: the reference's PK_CACHE (transient-crypto/src/proofs.rs:408-470,
    an LRU of 5 keys keyed by the persistent hash of the key bytes).
    params_for(k) gives the SRS of size 2^k (from_srs: the server's largest
    SRS downsized, params.rs:60-77, each size built once)."""

    def __init__(self, params_for, capacity=5, backend_factory=GpuBackend):
        self.params_for = params_for
        self.capacity = capacity
        self.backend_factory = backend_factory
        self._keys = collections.OrderedDict()
        self._lock = threading.Lock()

    @classmethod
    def from_srs(cls, srs, capacity=5, backend_factory=GpuBackend):
        sizes = {srs.k: srs}

        def params_for(k):
            if k > srs.k:
                raise ValueError("key needs a larger SRS than the server holds")
            if k not in sizes:
                sizes[k] = srs.downsize(k)
            return sizes[k]
        return cls(params_for, capacity, backend_factory)

    def get(self, key_id, key_bytes=None):
        """(params, pk, backend) of a key, building it from key_bytes when it
        is not held; raises KeyError for an unknown key sent without bytes"""
        from .keyfile import parse_pk, read_pk
        with self._lock:
            if key_id in self._keys:
                self._keys.move_to_end(key_id)
                return self._keys[key_id]
            if key_bytes is None:
                raise KeyError("unknown proving key and no key material in the request")
            params = self.params_for(parse_pk(key_bytes)[0].k)
            backend = self.backend_factory(params)
            entry = (params, read_pk(key_bytes, params, backend), backend)
            self._keys[key_id] = entry
            while len(self._keys) > self.capacity:
                self._keys.popitem(last=False)
            return entry

    def __len__(self):
        return len(self._keys)


class CommitBatcher:
    """Commitments of the proofs in flight, fused into shared launches.

    A proof's commitment calls (advice, lookup, product, quotient and
    opening commitments, each a batch of MSMs over one SRS basis) come here
    instead of running on the proof's own lane.  A dispatcher thread, on a
    lane of its own, takes what is waiting once every running proof is
    waiting here or `window_s` after the first request, whichever comes
    first; groups the requests by basis (the same SRS size and Lagrange or
    coefficient form); concatenates each group's scalar vectors on the
    device; and runs the group as ONE ragged batch through the basis's
    resident context: every stage of the MSM engine (recode, sort,
    accumulation, fix-up, reduction) is one launch for all the proofs'
    MSMs.  The reference fans a context batch out over up to 16 host threads
    with an engine each (midnight-sppark-msm/src/bls12_381_g1_msm.cu:
    172-215); here the batch is one launch per stage.  Results are split
    back in request order, so each proof's bytes are unchanged."""

    def __init__(self, server, lane, window_s=0.0005):
        self.server = server
        self.window_s = window_s
        self._cv = threading.Condition()
        self._pending = []
        self._stop = False
        self.batches = 0
        self.fused_requests = 0
        self._lane = lane
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()

    def commit(self, params, lagrange, h, n, count):
        fut = Future()
        with self._cv:
            self._pending.append((params, lagrange, h, n, count, fut))
            self._cv.notify_all()
        return fut.result()

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        self._thread.join()

    def _take(self):
        with self._cv:
            while not self._pending and not self._stop:
                self._cv.wait()
            if not self._pending:
                return None
            deadline = time.perf_counter() + self.window_s
            while not self._stop:
                if len(self._pending) >= max(1, self.server.running()):
                    break
                left = deadline - time.perf_counter()
                if left <= 0:
                    break
                self._cv.wait(left)
            batch, self._pending = self._pending, []
            return batch

    def _run(self):
        from .kzg import affine_from_projective_batch
        if self.server._set_lane is not None:
            self.server._set_lane(self._lane)
        while True:
            batch = self._take()
            if batch is None:
                return
            groups = collections.OrderedDict()
            for req in batch:
                groups.setdefault((id(req[0]), req[1]), []).append(req)
            for reqs in groups.values():
                try:
                    params, lagrange = reqs[0][0], reqs[0][1]
                    ctx = params.context(lagrange)
                    if len(reqs) == 1:
                        _, _, h, n, count, fut = reqs[0]
                        res = ctx.device_batch(h, 0, n, count)
                    else:
                        vec = api.Bls12_381FrDeviceVec.concat_many_host([r[2] for r in reqs],
                                                                       np.zeros((0, 4), np.uint64))
                        slices, off = [], 0
                        for _, _, h, n, count, _ in reqs:
                            slices += [(off + i * n, 0, n) for i in range(count)]
                            off += h.len
                        res = ctx.device_ragged(vec, slices)
                        vec.free()
                    pts = affine_from_projective_batch(res)
                    at = 0
                    for _, _, _, _, count, fut in reqs:
                        fut.set_result(list(pts[at:at + count]))
                        at += count
                    self.batches += 1
                    self.fused_requests += len(reqs)
                except BaseException as e:  # every waiting proof sees the failure
                    for r in reqs:
                        if not r[5].done():
                            r[5].set_exception(e)


class FusedCommitBackend(GpuBackend):
    """GpuBackend whose commitments go through a CommitBatcher."""

    def __init__(self, params, batcher):
        super().__init__(params)
        self.batcher = batcher

    def _commit(self, h, n, count, lagrange):
        return self.batcher.commit(self.params, lagrange, h, n, count)

    def commit_async(self, h, n, count, lagrange):
        return _ReadyPoints(self._commit(h, n, count, lagrange))


class _ReadyPoints:
    def __init__(self, points):
        self.points = points

    def result(self):
        return self.points


class ProofServer:
    """entries: {circuit_id: (params, pk)}; slots: proofs in flight;
    hbm_budget: bytes the proofs in flight may hold together (None = no
    limit beyond the slots)."""

    def __init__(self, entries, slots=4, hbm_budget=None, backend_factory=GpuBackend, lane_base=1,
                 set_lane=api.execution_lane_set, keystore=None, fuse_commits=False, lockstep=1):
        self.entries = entries
        # lockstep > 1: a worker takes up to that many waiting requests of
        # one circuit and proves them together (plonk.create_proofs): each
        # round's commitments of all of them are one MSM batch
        self.lockstep = max(1, int(lockstep))
        self.keystore = keystore
        self.slots = slots
        self.budget = hbm_budget
        self._set_lane = set_lane
        self._running = 0
        self._cv = threading.Condition()
        # fuse_commits: the proofs' commitments run as shared batches on a
        # lane of their own (CommitBatcher)
        self.batcher = CommitBatcher(self, lane_base + slots) if fuse_commits else None
        if self.batcher is not None:
            backend_factory = lambda params: FusedCommitBackend(params, self.batcher)  # noqa: E731
        self.backends = {cid: backend_factory(params) for cid, (params, _) in entries.items()}
        for params, _ in entries.values():
            if hasattr(params, "context"):
                params.context(True)
                params.context(False)
        self._pending = collections.deque()
        self._in_use = 0
        self.peak_in_use = 0
        self.peak_running = 0
        self._stop = False
        self.completed = []
        self._workers = [threading.Thread(target=self._worker, args=(lane_base + i,), daemon=True)
                         for i in range(slots)]
        for t in self._workers:
            t.start()

    def running(self):
        """proofs on a worker now"""
        return self._running

    def submit(self, circuit_id, witness, seed):
        params, pk = self.entries[circuit_id]
        return self._submit(circuit_id, params, pk, self.backends[circuit_id], witness, seed)

    def handle(self, request):
        """The /prove request loop (proof-server/src/endpoints.rs:246-343): a
        tagged ProveRequest (wire.py) in, the tagged proof out.  The key is
        the one the request carries or names, resolved through the key
        store; the proof runs on a lane like any submitted request."""
        from . import wire
        key_bytes, key_id, witness, seed = wire.decode_request(request)
        if self.keystore is None:
            raise ValueError("this server holds no key store for /prove requests")
        params, pk, backend = self.keystore.get(key_id, key_bytes)
        req = self._submit(key_id, params, pk, backend, witness, seed)
        return wire.encode_response(req.future.result())

    def _submit(self, circuit_id, params, pk, backend, witness, seed):
        req = Request(circuit_id, witness, seed, proof_footprint_bytes(pk.circuit), params, pk, backend)
        if self.budget is not None and req.bytes > self.budget:
            raise ValueError("request needs more device memory than the whole budget")
        with self._cv:
            self._pending.append(req)
            self._cv.notify_all()
        return req

    def _take(self):
        """the oldest pending request that fits in the budget left, with up
        to lockstep - 1 later requests for the same key that also fit"""
        for i, req in enumerate(self._pending):
            if self.budget is None or self._in_use + req.bytes <= self.budget:
                del self._pending[i]
                group, used = [req], req.bytes
                if self.lockstep > 1:
                    for other in list(self._pending):
                        if len(group) == self.lockstep:
                            break
                        if other.pk is req.pk and other.backend is req.backend and (
                                self.budget is None or self._in_use + used + other.bytes <= self.budget):
                            self._pending.remove(other)
                            group.append(other)
                            used += other.bytes
                return group
        return None

    def _worker(self, lane):
        if self._set_lane is not None:
            self._set_lane(lane)
        while True:
            with self._cv:
                while True:
                    if self._stop and not self._pending:
                        return
                    group = self._take()
                    if group is not None:
                        break
                    self._cv.wait()
                size = sum(r.bytes for r in group)
                self._in_use += size
                self._running += len(group)
                self.peak_in_use = max(self.peak_in_use, self._in_use)
                self.peak_running = max(self.peak_running, self._running)
            try:
                start = time.perf_counter()
                for r in group:
                    r.start = start
                first = group[0]
                if len(group) == 1:
                    proofs = [create_proof(first.params, first.pk, first.witness, first.backend,
                                           CircuitTranscript(), ChaCha20Rng.from_label(first.seed))]
                else:
                    proofs = create_proofs(first.params, first.pk, [r.witness for r in group], first.backend,
                                           [CircuitTranscript() for _ in group],
                                           [ChaCha20Rng.from_label(r.seed) for r in group])
                finish = time.perf_counter()
                for r, proof in zip(group, proofs):
                    r.proof, r.finish = proof, finish
                    r.future.set_result(proof)
            except BaseException as e:  # the group fails, the server keeps serving
                finish = time.perf_counter()
                for r in group:
                    r.finish = finish
                    if not r.future.done():
                        r.future.set_exception(e)
            finally:
                with self._cv:
                    self._in_use -= size
                    self._running -= len(group)
                    self.completed.extend(group)
                    self._cv.notify_all()

    def drain(self):
        """wait until nothing is pending or running"""
        with self._cv:
            while self._pending or self._running:
                self._cv.wait()

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._workers:
            t.join()
        if self.batcher is not None:
            self.batcher.close()


def poisson_arrivals(rng, rate, count):
    """arrival offsets (seconds) of a Poisson stream; rng a numpy Generator"""
    gaps = rng.exponential(1.0 / rate, size=count)
    out, t = [], 0.0
    for g in gaps:
        t += g
        out.append(t)
    return out


def run_stream(server, requests, arrivals):
    """Submit (circuit_id, witness, seed) requests at the given offsets from
    now; returns the finished Request objects in submission order."""
    t0 = time.perf_counter()
    subs = []
    for (cid, wit, seed), at in zip(requests, arrivals):
        delay = t0 + at - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        req = server.submit(cid, wit, seed)
        req.arrival = t0 + at
        subs.append(req)
    for r in subs:
        r.future.exception()
    return subs, t0


def latency_summary(reqs, t0):
    lat = sorted((r.finish - r.arrival) for r in reqs)
    span = max(r.finish for r in reqs) - t0
    pct = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))]  # noqa: E731
    return {"proofs": len(reqs), "proofs_per_s": len(reqs) / span, "p50_ms": pct(0.5) * 1e3,
            "p99_ms": pct(0.99) * 1e3, "mean_ms": sum(lat) / len(lat) * 1e3, "makespan_s": span}
