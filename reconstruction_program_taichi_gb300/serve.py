"""Reconstruction serving loop on one GPU: continuous admission, same-geometry
batching, captured CUDA graphs, p50/p99 latency.

No counterpart in the reference (it reconstructs one config at a time).

Model
  * A request is an FBP/FDK reconstruction or an N-iteration CGLS solve of one
    sinogram for one geometry (a parsed config).
  * Requests of the same kind, storage precision (and CGLS iteration count) whose
    parsed configs agree in every attribute that can change the result (a digest of
    the whole parsed config, file names aside) share a *slot class*.  A slot owns
    device buffers for up to `batch` requests, a CUDA stream, and one CUDA graph per
    member captured once (weight -> filter -> pack -> backproject of its sinogram, or its
    whole CGLS solve), so a batch of k requests executes as k graph launches and runs
    exactly k reconstructions.
  * Admission is continuous: a scheduler thread takes pending requests in arrival
    order, groups those whose slot class matches (up to `batch`), and starts them on
    a free slot; new slots are created while the HBM budget allows, and a slot is
    reused as soon as its previous batch finishes.  A new slot is built by the worker
    thread of its first batch, outside the scheduler's lock (one slot at a time, since a
    graph capture cannot overlap another thread's).  Batches on different slots run
    concurrently on their own streams.
  * Slots are kept for reuse; when a request needs a new slot and the budget is
    spent, idle slots of other classes are evicted, least recently used first.
  * Inputs may be host arrays or CUDA tensors already resident on the device; the
    result comes back in the same form (a new device tensor for device inputs, so
    resident data never crosses the host link).  Inputs may also be file paths, read
    with the reference's conventions for the request's config on the server's I/O
    threads from the moment of submission; a request is admitted only once its
    inputs are in memory, so disk reads overlap the GPU work of other requests.  With
    `out_path` the result is also written there on an I/O thread after its slot has
    been released; the future resolves once the file is written.
  * Results do not depend on the mix: every kernel is deterministic and a slot's
    graph always runs the same kernels on the same buffer layout.
"""
import os
import threading
import time
from concurrent.futures import Future, ThreadPoolExecutor

import numpy as np
import torch

from . import ops
from .fbp import FdkPipeline
from .io import imwriteRaw, read_sinogram_file

# Parsed-config attributes that only name files or control logging: they do not
# change what a slot computes, so requests that differ only in them share a slot.
_IO_ONLY = frozenset({
    "config_dict", "input_dir", "output_dir", "input_files_pattern", "output_file_prefix",
    "output_file_replace", "output_file_format", "input_file_form", "save_filtered_sinogram",
    "verbose", "input_path", "output_path", "output_file", "img_sgm", "img_recon", "img_x",
    "file_processed_count", "num_iter_runned", "loss", "prior_image_file", "img_prior",
})


def _digest_value(h, v):
    if isinstance(v, np.ndarray):
        a = np.ascontiguousarray(v)
        h.update(f"nd{a.dtype.str}{a.shape}".encode())
        h.update(a.tobytes())
    elif isinstance(v, (list, tuple)):
        h.update(f"seq{len(v)}[".encode())
        for x in v:
            _digest_value(h, x)
        h.update(b"]")
    elif isinstance(v, dict):
        h.update(f"map{len(v)}{{".encode())
        for k in sorted(v, key=repr):
            h.update(repr(k).encode())
            _digest_value(h, v[k])
        h.update(b"}")
    else:  # scalars (float repr is exact), strings, None
        h.update(f"{type(v).__name__}:{v!r};".encode())


def config_digest(obj):
    """Digest of every parsed-config attribute that can change a reconstruction:
    every attribute of the parsed object except the file-naming and logging ones
    (_IO_ONLY) and private caches; arrays (angles, projection matrices, beam-hardening
    coefficients, per-view centres) by their bytes.  Two configs with the same digest
    produce the same result from the same sinogram."""
    import hashlib
    h = hashlib.sha256()
    for k in sorted(vars(obj)):
        if k.startswith("_") or k in _IO_ONLY:
            continue
        v = getattr(obj, k)
        if callable(v):
            continue
        h.update(k.encode() + b"=")
        _digest_value(h, v)
    return h.hexdigest()


def _geom_key(obj, kind, extra=()):
    """Slot class of a request: its kind, the digest of its parsed config and the
    per-request options (storage, iteration count)."""
    return (kind, config_digest(obj)) + tuple(extra)


def _is_path(a):
    return isinstance(a, (str, os.PathLike))


def _input_error(r):
    """The exception of a failed input read of request r, else None."""
    for a in (r.sgm, r.x0):
        if isinstance(a, Future) and a.done() and a.exception() is not None:
            return a.exception()
    return None


def _inputs_ready(r):
    return all(not isinstance(a, Future) or a.done() for a in (r.sgm, r.x0))


def _resolve_inputs(r):
    if isinstance(r.sgm, Future):
        r.sgm = r.sgm.result()
    if isinstance(r.x0, Future):
        r.x0 = r.x0.result()


def _to_device(a, device):
    """A host array or a tensor as a float32 tensor on device (no copy when it already is)."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.float32)
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(device)


class _Request:
    __slots__ = ("kind", "obj", "sgm", "x0", "n_iter", "storage", "key", "future", "t_arrive", "t_start",
                 "t_done", "units", "on_device", "out_path")

    def __init__(self, kind, obj, sgm, x0=None, n_iter=0, storage="f32", out_path=None):
        self.kind, self.obj, self.sgm, self.x0, self.n_iter, self.storage = kind, obj, sgm, x0, n_iter, storage
        self.out_path = out_path
        extra = (storage, n_iter) if kind == "cgls" else (storage,)
        self.key = _geom_key(obj, kind, extra)
        self.future = Future()
        self.t_arrive = time.perf_counter()
        self.t_start = self.t_done = None
        nvox = obj.img_dim * obj.img_dim * obj.img_dim_z
        self.units = nvox * obj.view_num * (1 if kind == "fbp" else 2 * (n_iter + 1))
        self.on_device = isinstance(sgm, torch.Tensor) and sgm.is_cuda


_IR_STORAGE = {"f32": "float32", "bf16": "bfloat16", "f16": "float16"}


def _capture_members(stream, bodies):
    """One CUDA graph per batch member: body(i) is run once on stream for its
    first-call set-up (cached buffers are created outside any capture), then every
    member's body is captured into its own graph.  The graphs draw on one memory pool,
    which is safe because a slot replays them one after another on its stream."""
    with torch.cuda.stream(stream):
        bodies[0]()
    stream.synchronize()
    pool = torch.cuda.graph_pool_handle()
    graphs = []
    for body in bodies:
        g = torch.cuda.CUDAGraph()
        # thread-local capture: other slots keep running on their own threads and streams
        with torch.cuda.graph(g, pool=pool, stream=stream, capture_error_mode="thread_local"):
            body()
        graphs.append(g)
    return graphs


class _FbpSlot:
    """Static buffers for `batch` FBP reconstructions of one slot class and one captured
    graph per member: a batch of k requests replays the graphs of its first k members,
    so no member recomputes a stale input.  The mixed-precision path (16-bit storage)
    uses the two-part tensor-core filter and 16-bit backprojection coefficients."""

    def __init__(self, obj, batch, storage, device, use_graph):
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.batch = batch
        impl = "tc3" if storage == "f32" else "tc"
        with torch.cuda.stream(self.stream):
            self.pipes = [FdkPipeline(obj, device=device, storage=storage, filter_impl=impl) for _ in range(batch)]
            shape = self.pipes[0].dg.sgm_shape
            self.inp = [torch.zeros(shape, dtype=torch.float32, device=device) for _ in range(batch)]
            self.out = [torch.zeros(self.pipes[0].dg.vol_shape, dtype=torch.float32, device=device)
                        for _ in range(batch)]
            # the pipelines' buffers and tensor-core filters (whose set-up kernel runs
            # here, on the slot's stream), before the slot counts its bytes
            for p in self.pipes:
                p.allocate()
        self.host_out = [torch.empty(self.pipes[0].dg.vol_shape, dtype=torch.float32, pin_memory=True)
                         for _ in range(batch)]
        self.graphs = []
        self.last_used = time.perf_counter()
        self.nbytes = sum(p.nbytes() for p in self.pipes) + sum(t.numel() * 4 for t in self.inp + self.out)
        if use_graph:
            self.graphs = _capture_members(self.stream, [lambda i=i: self._member(i) for i in range(batch)])

    def _member(self, i):
        self.pipes[i].run(self.inp[i], out=self.out[i])

    def run(self, reqs, done=None):
        """Reconstruct reqs (at most `batch`); returns their results in order.  done(i,
        result), when given, is called for every member but the last as soon as that
        member's result is ready."""
        pending = []
        with torch.cuda.stream(self.stream):
            for i, r in enumerate(reqs):
                if r.on_device:
                    self.inp[i].copy_(r.sgm)
                else:
                    self.inp[i].copy_(torch.from_numpy(np.ascontiguousarray(r.sgm, dtype=np.float32)))
                if self.graphs:
                    self.graphs[i].replay()
                else:
                    self._member(i)
                if r.on_device:
                    res = self.out[i].clone()
                else:
                    res = None
                    self.host_out[i].copy_(self.out[i], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(self.stream)
                pending.append((ev, res))
        outs = []
        for i, (ev, res) in enumerate(pending):
            ev.synchronize()
            out = res if res is not None else self.host_out[i].numpy().copy()
            if done is not None and i + 1 < len(pending):
                done(i, out)
            outs.append(out)
        self.last_used = time.perf_counter()
        return outs


def _fp_workspace_bytes(dg, dtype):
    from . import _lib
    return int(_lib.load().mct_fp_storage_workspace_size(dg.g(), int(dtype)))


class _CglsSlot:
    """n_iter CGLS iterations (reference operator pair, lambda * D^T D with unit
    weights, as submit_cgls describes) for up to `batch` requests of one slot class.
    The members share one IrSystem (geometry tables, effective ray map, projector
    workspace, packed operand), which is safe because they run one after another on
    the slot's stream; each member has static input and output buffers and its own
    captured graph of the whole solve, so a batch of k requests is k graph launches."""

    def __init__(self, obj, n_iter, storage, batch, device, use_graph):
        from .ir import IrSystem
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.batch = batch
        self.obj = obj
        self.n_iter = n_iter
        self.lr = obj.coef_lambda * obj.pixel_count_ratio
        with torch.cuda.stream(self.stream):
            self.sys = IrSystem(obj, device, storage=_IR_STORAGE.get(storage, storage))
            dg = self.sys.dg
            f32 = dict(dtype=torch.float32, device=device)
            self.sgm = [torch.zeros(dg.sgm_shape, **f32) for _ in range(batch)]
            self.x0 = [torch.zeros(dg.vol_shape, **f32) for _ in range(batch)]
            self.out = [torch.zeros(dg.vol_shape, **f32) for _ in range(batch)]
            self.wr = torch.ones(dg.vol_shape, **f32)
        self.last_used = time.perf_counter()
        nvol = 4 * obj.img_dim * obj.img_dim * obj.img_dim_z
        nsgm = 4 * self.sys.fp_buf.numel()
        # per member: sinogram, seed, result; shared: unit weights, map, projector
        # buffer and workspace, packed operands (float32 and storage type), and the
        # temporaries of one solve (masked sinogram, P^T b, d, r, x, q)
        self.nbytes = (batch * (nsgm + 2 * nvol) + nvol + 2 * nsgm + _fp_workspace_bytes(dg, self.sys.fp_dtype)
                       + 2 * 4 * nsgm + nsgm + 5 * nvol)
        self.graphs = []
        if use_graph:
            self.graphs = _capture_members(self.stream, [lambda i=i: self._member(i) for i in range(batch)])

    def _member(self, i):
        sy = self.sys
        sy.bpb = sy.bp_b(self.sgm[i])
        x = sy.cgls(self.x0[i], [], [(self.lr, self.wr)], self.n_iter)
        self.out[i].copy_(x)

    def run(self, reqs, done=None):
        """As _FbpSlot.run: results in order, done(i, result) early for all but the last."""
        pending = []
        with torch.cuda.stream(self.stream):
            for i, r in enumerate(reqs):
                self.sgm[i].copy_(_to_device(r.sgm, self.device))
                self.x0[i].copy_(_to_device(r.x0, self.device))
                if self.graphs:
                    self.graphs[i].replay()
                else:
                    self._member(i)
                res = self.out[i].clone()
                ev = torch.cuda.Event()
                ev.record(self.stream)
                pending.append((ev, res, r.on_device))
        outs = []
        for i, (ev, res, on_device) in enumerate(pending):
            ev.synchronize()
            out = res if on_device else res.cpu().numpy()
            if done is not None and i + 1 < len(pending):
                done(i, out)
            outs.append(out)
        self.last_used = time.perf_counter()
        return outs


class ReconServer:
    """Continuous-batching reconstruction server on one GPU (see module docstring)."""

    def __init__(self, device=None, hbm_budget_gb=150.0, batch=4, max_slots_per_class=4, use_graphs=True):
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required")
        self.device = torch.device(device or "cuda")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.budget = int(hbm_budget_gb * 1e9)
        self.used = 0
        self.batch = batch
        self.max_slots = max_slots_per_class
        self.use_graphs = use_graphs
        self.pending = []
        self.cv = threading.Condition()
        self.free_slots = {}    # key -> [slot]
        self.all_slots = {}     # key -> count (built and being built)
        self.evictions = 0
        self.busy = 0
        self.done = []
        self.closed = False
        self.errors = []
        self._workers = []
        # slot construction (buffers, warm-up, graph capture) runs on the workers,
        # outside self.cv, one slot at a time: a capture begins with a device-wide
        # synchronize, which is illegal while another thread is capturing
        self._build_lock = threading.Lock()
        self._io = ThreadPoolExecutor(2, thread_name_prefix="mct-serve-io")
        self._thread = threading.Thread(target=self._schedule, daemon=True)
        self._thread.start()

    # ------------------------------------------------------------ API
    def submit_fbp(self, obj, sgm, storage="f32", out_path=None):
        """FBP/FDK of a sinogram [rows, views, cols] (host array, CUDA tensor, or the path
        of an input file in the config's InputFileForm and detector row range) for the
        parsed config obj; the future's result is a host array or a new CUDA tensor.
        storage: 'f32' (plain) or 'bf16' / 'f16' (mixed precision: two-part tensor-core
        filter, 16-bit backprojection operand).  out_path: also write the result there
        (raw float32)."""
        sgm = self._load(sgm, lambda p: read_sinogram_file(obj, p))
        return self._submit(_Request("fbp", obj, sgm, storage=storage, out_path=out_path))

    def submit_cgls(self, obj, sgm, x0, n_iter, storage="f32", out_path=None):
        """n_iter CGLS iterations (Tikhonov-TV with unit weights) from x0 (host arrays,
        CUDA tensors or file paths as for submit_fbp; a volume file is raw float32
        [z, y, x]).  storage: 'f32', or 'bf16' / 'f16' for 16-bit projector gathers
        inside the iterations (the data term stays float32)."""
        sgm = self._load(sgm, lambda p: read_sinogram_file(obj, p))
        x0 = self._load(x0, lambda p: np.fromfile(p, dtype=np.float32).reshape(obj.img_dim_z, obj.img_dim,
                                                                             obj.img_dim))
        return self._submit(_Request("cgls", obj, sgm, x0=x0, n_iter=n_iter, storage=storage, out_path=out_path))

    def close(self, wait=True):
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        if wait:
            self._thread.join()
            for t in self._workers:
                t.join()
        self._io.shutdown(wait=wait)  # pending result writes finish first when waiting

    def stats(self):
        """Latency (arrival to result), its queueing and service parts, throughput."""
        done = list(self.done)
        lat = np.array([(r.t_done - r.t_arrive) * 1e3 for r in done]) if done else np.zeros(1)
        wait = np.array([(r.t_start - r.t_arrive) * 1e3 for r in done]) if done else np.zeros(1)
        serv = np.array([(r.t_done - r.t_start) * 1e3 for r in done]) if done else np.zeros(1)
        t0 = min(r.t_arrive for r in done) if done else 0.0
        t1 = max(r.t_done for r in done) if done else 1.0
        units = sum(r.units for r in done)
        slots = {}
        for k, v in self.all_slots.items():
            slots[k[0]] = slots.get(k[0], 0) + v
        return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "queue_p50_ms": float(np.percentile(wait, 50)), "service_p50_ms": float(np.percentile(serv, 50)),
                "service_p99_ms": float(np.percentile(serv, 99)),
                "gups": units / max(t1 - t0, 1e-9) / 1e9, "slots": slots, "classes": len(self.all_slots),
                "evictions": self.evictions, "hbm_used_gb": self.used / 1e9}

    # ------------------------------------------------------------ internals
    def _load(self, a, reader):
        """A path becomes a future of its contents, read on an I/O thread; the scheduler
        is woken when the read ends."""
        if not _is_path(a):
            return a
        fut = self._io.submit(reader, os.fspath(a))
        fut.add_done_callback(self._wake)
        return fut

    def _wake(self, _fut=None):
        with self.cv:
            self.cv.notify_all()

    def _write_result(self, r, out):
        try:
            imwriteRaw(out.cpu().numpy() if isinstance(out, torch.Tensor) else out, os.fspath(r.out_path),
                       dtype=np.float32)
            r.future.set_result(out)
        except Exception as e:  # noqa: BLE001 - handed to the caller through the future
            r.future.set_exception(e)

    def _submit(self, req):
        with self.cv:
            if self.closed:
                raise RuntimeError("server is closed")
            self.pending.append(req)
            self.cv.notify_all()
        return req.future

    def _make_slot(self, req):
        torch.cuda.set_device(self.device)
        with self._build_lock:
            if req.kind == "fbp":
                return _FbpSlot(req.obj, self._batch_for(req), req.storage, self.device, self.use_graphs)
            return _CglsSlot(req.obj, req.n_iter, req.storage, self._batch_for(req), self.device, self.use_graphs)

    @staticmethod
    def _per_request_bytes(req):
        o = req.obj
        nvol = o.img_dim * o.img_dim * o.img_dim_z * 4
        nsgm = o.det_elem_count_horizontal * o.det_elem_count_vertical_actual * o.view_num * 4
        if req.kind == "fbp":  # input, filtered, packed (4x), tensor-core operand tiles (1.5x), bound
            return nsgm * 8 + 2 * nvol
        # CGLS member: sinogram, seed, result
        return nsgm + 2 * nvol

    @staticmethod
    def _shared_bytes(req):
        """Bytes a slot holds whatever its batch (CGLS: the shared IrSystem and the
        temporaries of one solve; FBP: none)."""
        if req.kind == "fbp":
            return 0
        o = req.obj
        nvol = o.img_dim * o.img_dim * o.img_dim_z * 4
        nsgm = o.det_elem_count_horizontal * o.det_elem_count_vertical_actual * o.view_num * 4
        # unit weights, map, projector buffer, gather copies (cone beam, float32 quad
        # copies: 8 floats per voxel), packed operands (2 x 4 per element), temporaries
        return nvol + 2 * nsgm + (8 if o.cone_beam else 1) * nvol + 8 * nsgm + nsgm + 5 * nvol

    def _batch_for(self, req):
        """Requests per slot: `batch`, reduced so that one slot takes at most an eighth
        of the budget (large geometries get small slots, so that several classes stay
        resident)."""
        per = max(self._per_request_bytes(req), 1)
        room = self.budget / 8 - self._shared_bytes(req)
        return max(1, min(self.batch, int(room // per)))

    def _estimate(self, req):
        return self._shared_bytes(req) + self._batch_for(req) * self._per_request_bytes(req)

    def _schedule(self):
        while True:
            with self.cv:
                while not self.closed and not self.pending:
                    self.cv.wait()
                if self.closed and not self.pending:
                    break
                started = self._try_start()
                if not started:
                    self.cv.wait(timeout=0.05)

    def _try_start(self):
        """Start the oldest pending request's class on a free slot, or reserve the
        budget for a new slot and hand its construction to the batch's worker (the
        slot is built outside the lock); returns True if something started.  Called
        with the lock held."""
        for i, head in enumerate(self.pending):
            err = _input_error(head)
            if err is not None:  # its input file could not be read: fail this request only
                head.future.set_exception(err)
                self.pending.pop(i)
                return True
            if not _inputs_ready(head):
                continue
            key = head.key
            free = self.free_slots.setdefault(key, [])
            slot = free.pop() if free else None
            reserved = 0
            if slot is None:
                if self.all_slots.get(key, 0) >= self.max_slots:
                    continue
                need = self._estimate(head)
                if self.used + need > self.budget:
                    self._evict_idle(need, keep=key)
                if self.used + need > self.budget:
                    if self.busy == 0 and not any(self.free_slots.values()):
                        head.future.set_exception(MemoryError("request exceeds the HBM budget"))
                        self.pending.pop(i)
                        return True
                    continue
                reserved = need
                self.used += need
                self.all_slots[key] = self.all_slots.get(key, 0) + 1
            cap = slot.batch if slot is not None else self._batch_for(head)
            group = [r for r in self.pending if r.key == key and _inputs_ready(r) and _input_error(r) is None]
            group = group[:cap]
            for r in group:
                self.pending.remove(r)
                r.t_start = time.perf_counter()
            self.busy += 1
            t = threading.Thread(target=self._run, args=(slot, key, group, reserved), daemon=True)
            self._workers.append(t)
            t.start()
            return True
        return False

    def _evict_idle(self, need, keep):
        """Release idle slots of other classes, least recently used first, until `need`
        bytes fit in the budget (called with the lock held)."""
        idle = [(s.last_used, k, s) for k, lst in self.free_slots.items() if k != keep for s in lst]
        for _, k, s in sorted(idle, key=lambda t: t[0]):
            if self.used + need <= self.budget:
                break
            self.free_slots[k].remove(s)
            self.all_slots[k] -= 1
            if self.all_slots[k] == 0:
                del self.all_slots[k]
            self.used -= s.nbytes
            self.evictions += 1
            del s

    def _run(self, slot, key, group, reserved):
        """Worker of one batch: builds the slot first when the scheduler reserved the
        budget for a new one (outside the lock, so finishing batches are not held up),
        then runs the batch and returns the slot."""
        outs, err, early = None, None, set()
        try:
            torch.cuda.set_device(self.device)
            if slot is None:
                try:
                    slot = self._make_slot(group[0])
                finally:
                    with self.cv:
                        if slot is None:  # construction failed: release the reservation
                            self.used -= reserved
                            self.all_slots[key] -= 1
                            if self.all_slots[key] == 0:
                                del self.all_slots[key]
                        else:  # account the slot's own size instead of the estimate
                            self.used += slot.nbytes - reserved
            for r in group:
                _resolve_inputs(r)
            early = set()

            def member_done(i, out):
                # a member before the batch's last: recorded, then delivered at once
                r = group[i]
                r.t_done = time.perf_counter()
                with self.cv:
                    self.done.append(r)
                early.add(i)
                self._deliver(r, out)

            outs = slot.run(group, member_done)
            now = time.perf_counter()
            for i, r in enumerate(group):
                if i not in early:
                    r.t_done = now
        except Exception as e:  # a failed batch fails its own requests only
            err = e
            self.errors.append(e)
        # record completion and free the slot before any caller can observe the last result
        with self.cv:
            if outs is not None:
                self.done.extend(r for i, r in enumerate(group) if i not in early)
            self.busy -= 1
            if slot is not None:
                self.free_slots.setdefault(key, []).append(slot)
            self.cv.notify_all()
        for i, r in enumerate(group):
            if outs is not None:
                if i not in early:
                    self._deliver(r, outs[i])
            elif not r.future.done():
                r.future.set_exception(err)

    def _deliver(self, r, out):
        """Resolve r's future with out (after writing out_path, on an I/O thread)."""
        if r.out_path is not None:
            try:
                self._io.submit(self._write_result, r, out)
            except RuntimeError:  # I/O threads already shut down (close without waiting)
                self._write_result(r, out)
        else:
            r.future.set_result(out)
