"""Learned inlier-probability proposal for the PROSAC sampler.

A per-correspondence MLP (k = 8 nearest-neighbour displacement features,
4 layers of width 128, BF16 weights and FP32 accumulation) scores how likely
each correspondence is an inlier; each pair's correspondences are reordered by
descending score and the engine runs its PROSAC sampler (sampler = 1) on that
order, which draws from the most promising correspondences first. The inlier
mask is mapped back to the caller's order. The reference has no such network:
its samplers 3 and 4 take externally computed probabilities
(src/pygcransac/src/bindings.cpp, `probabilities`); this module produces the
order from the correspondences alone, and `predict` gives probabilities that
the importance sampler (sampler 3) of the entry points accepts.

The features, forward pass, backward pass, Adam update, ordering and mask
mapping are the engine's own kernels (csrc/gcr_learned.cu, reached through the
C-ABI); torch only provides device buffers, streams and graphs.

Training data: inlier masks that the plain method (this engine, uniform
sampler) produces on synthetic scenes; `train_proposal.py` is the recipe.
"""
import ctypes
import json
import struct

import numpy as np

from . import _abi

MAGIC = b"GCRL"


def _torch():
    import torch
    return torch


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _check(rc, where):
    if rc != _abi.GCR_OK:
        raise RuntimeError(f"{where}: {_abi.last_error()}")


def layout(P):
    """(offsets [P+1] int64, max_n, pair_of_row [total] int32) of pair sizes P."""
    lens = np.asarray(P, np.int64)
    offsets = np.zeros(len(lens) + 1, np.int64)
    offsets[1:] = np.cumsum(lens)
    return offsets, int(lens.max()) if len(lens) else 0, np.repeat(np.arange(len(lens), dtype=np.int32), lens)


class LearnedProposal:
    """Network parameters (FP32 master + BF16 copy), Adam state, training and
    inference."""

    def __init__(self, seed=0, device="cuda"):
        torch = _torch()
        self.lib = _abi.load()
        self.device = device
        self.count = int(self.lib.gcr_learned_param_count())
        self.width = int(self.lib.gcr_learned_feature_width())
        rng = np.random.Generator(np.random.PCG64(seed))
        P = np.zeros(self.count, np.float32)
        # He-uniform weights, zero biases
        off = 0
        for fan_in, fan_out in [(self.width, 128), (128, 128), (128, 128), (128, 1)]:
            bound = np.sqrt(6.0 / fan_in)
            P[off:off + fan_in * fan_out] = rng.uniform(-bound, bound, fan_in * fan_out)
            off += fan_in * fan_out + fan_out
        self.master = torch.from_numpy(P).to(device)
        self.bf16 = torch.zeros(self.count, dtype=torch.bfloat16, device=device)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.grad = torch.zeros_like(self.master)
        self.step = 0
        self.info = {}
        self._refresh()

    def _refresh(self):
        _check(self.lib.gcr_learned_params_to_bf16(_ptr(self.master), _ptr(self.bf16), None), "params_to_bf16")

    # -------------------------------------------------------------- parameters
    def parameters(self):
        return self.master.cpu().numpy().copy()

    def load_parameters(self, P):
        torch = _torch()
        self.master.copy_(torch.from_numpy(np.ascontiguousarray(P, np.float32)))
        self._refresh()

    def bf16_parameters(self):
        """The BF16 weights the kernels read, as float64."""
        return self.bf16.float().cpu().numpy().astype(np.float64)

    def save(self, path, info=None):
        """Checkpoint: MAGIC, u32 header length, JSON header, then the FP32
        master parameters and the Adam moments (float32, little-endian)."""
        hdr = dict(self.info, **(info or {}))
        hdr.update(count=self.count, feature_width=self.width, step=self.step)
        hb = json.dumps(hdr, sort_keys=True).encode()
        with open(path, "wb") as f:
            f.write(MAGIC + struct.pack("<I", len(hb)) + hb)
            for t in (self.master, self.m, self.v):
                f.write(t.cpu().numpy().astype("<f4").tobytes())

    @classmethod
    def load(cls, path, device="cuda"):
        torch = _torch()
        with open(path, "rb") as f:
            blob = f.read()
        if blob[:4] != MAGIC:
            raise ValueError(f"{path}: not a learned-proposal checkpoint")
        (hl,) = struct.unpack("<I", blob[4:8])
        hdr = json.loads(blob[8:8 + hl].decode())
        self = cls(device=device)
        if hdr["count"] != self.count or hdr["feature_width"] != self.width:
            raise ValueError(f"{path}: parameter layout {hdr['count']}/{hdr['feature_width']} does not match "
                             f"{self.count}/{self.width}")
        arr = np.frombuffer(blob[8 + hl:], "<f4")
        if len(arr) != 3 * self.count:
            raise ValueError(f"{path}: truncated")
        self.master.copy_(torch.from_numpy(arr[:self.count].copy()))
        self.m.copy_(torch.from_numpy(arr[self.count:2 * self.count].copy()))
        self.v.copy_(torch.from_numpy(arr[2 * self.count:].copy()))
        self.step = int(hdr["step"])
        self.info = {k: v for k, v in hdr.items() if k not in ("count", "feature_width", "step")}
        self._refresh()
        return self

    # ---------------------------------------------------------------- features
    def features(self, d_corr, d_offsets, d_sizes, num_pairs, max_n, total):
        """Device features [total, width] of pairs already on the device."""
        torch = _torch()
        feat = torch.empty((total, self.width), dtype=torch.float32, device=self.device)
        _check(self.lib.gcr_learned_features(_ptr(d_corr), _ptr(d_offsets), _ptr(d_sizes), num_pairs, max_n,
                                             _ptr(feat), None), "features")
        return feat

    def upload(self, corr_list, sizes):
        """(d_corr, d_offsets, d_sizes, offsets, max_n, pair_of_row) of host pairs."""
        torch = _torch()
        offsets, max_n, por = layout([len(c) for c in corr_list])
        d_corr = torch.from_numpy(np.ascontiguousarray(np.concatenate(corr_list), np.float64)).to(self.device)
        d_off = torch.from_numpy(offsets).to(self.device)
        d_sz = torch.from_numpy(_sizes(sizes).view(np.int32).copy()).to(self.device)
        return d_corr, d_off, d_sz, offsets, max_n, por

    def host_features(self, corr_list, sizes):
        d_corr, d_off, d_sz, offsets, max_n, _ = self.upload(corr_list, sizes)
        return self.features(d_corr, d_off, d_sz, len(corr_list), max_n, int(offsets[-1])), offsets

    # --------------------------------------------------------------- inference
    def logits(self, feat):
        torch = _torch()
        n = feat.shape[0]
        z = torch.empty(n, dtype=torch.float32, device=self.device)
        _check(self.lib.gcr_learned_forward(_ptr(feat), n, _ptr(self.bf16), None, None, None, _ptr(z), None),
               "forward")
        return z

    def predict(self, corr_list, sizes):
        """Inlier probabilities, one array per pair."""
        torch = _torch()
        feat, offsets = self.host_features(corr_list, sizes)
        p = torch.sigmoid(self.logits(feat)).cpu().numpy()
        return [p[offsets[i]:offsets[i + 1]] for i in range(len(corr_list))]

    # ---------------------------------------------------------------- training
    def loss_and_grad(self, feat, labels, weights):
        """Weighted BCE (divided by the weight sum) and its gradient (device)."""
        torch = _torch()
        n = feat.shape[0]
        a1 = torch.empty((n, 128), dtype=torch.float32, device=self.device)
        a2 = torch.empty_like(a1)
        a3 = torch.empty_like(a1)
        z = torch.empty(n, dtype=torch.float32, device=self.device)
        _check(self.lib.gcr_learned_forward(_ptr(feat), n, _ptr(self.bf16), _ptr(a1), _ptr(a2), _ptr(a3), _ptr(z),
                                            None), "forward")
        ws = float(weights.sum().item())
        self.grad.zero_()
        _check(self.lib.gcr_learned_backward(_ptr(feat), n, _ptr(self.bf16), _ptr(a1), _ptr(a2), _ptr(a3), _ptr(z),
                                             _ptr(labels), _ptr(weights), 1.0 / ws, _ptr(self.grad), None),
               "backward")
        loss = (weights * (torch.clamp(z, min=0) - z * labels + torch.log1p(torch.exp(-z.abs())))).sum() / ws
        return float(loss.item()), self.grad

    def adam(self, lr):
        self.step += 1
        _check(self.lib.gcr_learned_adam(_ptr(self.m), _ptr(self.v), _ptr(self.master), _ptr(self.bf16),
                                         _ptr(self.grad), float(lr), self.step, None), "adam")

    def train_rows(self, feat, labels, epochs=1, lr=1e-3, batch_rows=65536, seed=0, max_pos_weight=20.0):
        """Adam on the weighted BCE of device rows (feat [n, width], labels [n]
        in {0, 1}); positives weighted by the negative/positive ratio of each
        batch (at most max_pos_weight). Returns the loss of every batch."""
        torch = _torch()
        g = torch.Generator(device="cpu")
        g.manual_seed(seed)
        n = feat.shape[0]
        history = []
        for _ in range(epochs):
            perm = torch.randperm(n, generator=g).to(self.device)
            for b0 in range(0, n, batch_rows):
                r = perm[b0:b0 + batch_rows]
                fb = feat.index_select(0, r).contiguous()
                yb = labels.index_select(0, r).contiguous()
                pos = float(yb.sum().item())
                pw = min(max_pos_weight, (len(r) - pos) / pos) if pos > 0 else 1.0
                wb = torch.where(yb > 0.5, torch.full_like(yb, pw), torch.ones_like(yb))
                loss, _ = self.loss_and_grad(fb, yb, wb)
                self.adam(lr)
                history.append(loss)
        return history


def _sizes(sizes):
    s = np.asarray(sizes)
    z = np.zeros(len(s), _abi.SIZE_DTYPE)
    z["h1"], z["w1"], z["h2"], z["w2"] = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    return z


class LearnedBatch:
    """A device-resident batch run with the learned order: features, forward
    pass and per-pair ordering, then the engine's PROSAC run on the ordered
    correspondences, then the mask mapped back. `launch(stream)` queues only
    kernels (no host work, no allocation), so it can be recorded into a CUDA
    graph after `prepare`."""

    def __init__(self, proposal, kind, d_corr, offsets, sizes, params, seeds=None, K=None, ctx=None,
                 lo_precision=_abi.GCR_LO_FP64):
        torch = _torch()
        self.lib = _abi.load()
        self.proposal = proposal
        self.P = len(offsets) - 1
        self.offsets = np.ascontiguousarray(offsets, np.int64)
        lens = np.diff(self.offsets)
        self.total = int(self.offsets[-1])
        self.max_n = int(lens.max()) if self.P else 0
        dev = proposal.device
        self.d_corr = d_corr
        self.d_off = torch.from_numpy(self.offsets).to(dev)
        self.sizes = _sizes(sizes)
        self.d_sz = torch.from_numpy(self.sizes.view(np.int32).copy()).to(dev)
        self.d_por = torch.from_numpy(np.repeat(np.arange(self.P, dtype=np.int32), lens)).to(dev)
        self.d_feat = torch.empty((self.total, proposal.width), dtype=torch.float32, device=dev)
        self.d_logits = torch.empty(self.total, dtype=torch.float32, device=dev)
        self.d_sorted = torch.empty((self.total, 4), dtype=torch.float64, device=dev)
        self.d_perm = torch.empty(self.total, dtype=torch.int32, device=dev)
        self.d_models = torch.zeros(self.P * 9, dtype=torch.float64, device=dev)
        self.d_sorted_masks = torch.zeros(self.total, dtype=torch.uint8, device=dev)
        self.d_masks = torch.zeros(self.total, dtype=torch.uint8, device=dev)
        self.d_stats = torch.zeros(self.P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.own_ctx = ctx is None
        self.ctx = ctypes.c_void_p() if ctx is None else ctx
        if self.own_ctx:
            _check(self.lib.gcr_context_create(ctypes.byref(self.ctx)), "context_create")
        # GCR_LO_FP32: the local optimisation's F fits in FP32 (the engine's
        # fast mode for throughput forms; GCR_LO_FP64 keeps the oracle's arithmetic)
        _check(self.lib.gcr_context_set_lo_precision(self.ctx, int(lo_precision)), "set_lo_precision")
        self.params = _abi.Params(**{f: getattr(params, f) for f, _ in params._fields_})
        self.params.sampler = 1
        self.seeds = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
        self.K = None if K is None else np.ascontiguousarray(K, np.float64)
        self.kind = kind

    def prepare(self):
        _check(self.lib.gcr_batch_prepare(self.ctx, self.kind, self.P, _ptr(self.d_sorted), _abi.ptr(self.offsets),
                                          _abi.ptr(self.K), _abi.ptr(self.sizes), ctypes.byref(self.params),
                                          _abi.ptr(self.seeds), _ptr(self.d_models), _ptr(self.d_sorted_masks),
                                          _ptr(self.d_stats)), "batch_prepare")

    def launch(self, stream=None):
        """Queues the whole batch on `stream` (a torch stream or None for the
        current one). Returns the number of kernels launched."""
        torch = _torch()
        s = (stream or torch.cuda.current_stream()).cuda_stream
        sp = ctypes.c_void_p(s)
        _check(self.lib.gcr_learned_propose(_ptr(self.d_corr), _ptr(self.d_off), _ptr(self.d_sz), self.P, self.max_n,
                                            self.total, _ptr(self.proposal.bf16), _ptr(self.d_feat),
                                            _ptr(self.d_logits), _ptr(self.d_sorted), _ptr(self.d_perm), sp),
               "learned_propose")
        _check(self.lib.gcr_batch_launch(self.ctx, sp), "batch_launch")
        engine = int(self.lib.gcr_last_launch_count())
        _check(self.lib.gcr_learned_unpermute_mask(_ptr(self.d_sorted_masks), _ptr(self.d_perm), _ptr(self.d_off),
                                                   _ptr(self.d_por), self.total, _ptr(self.d_masks), sp),
               "unpermute_mask")
        return 3 + engine + 1

    def results(self):
        """(models [P, 3, 3], masks list of bool arrays, stats) on the host."""
        models = self.d_models.cpu().numpy().reshape(self.P, 3, 3)
        m = self.d_masks.cpu().numpy().astype(bool)
        stats = np.frombuffer(self.d_stats.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
        return models, [m[self.offsets[i]:self.offsets[i + 1]] for i in range(self.P)], stats

    def close(self):
        if self.own_ctx and self.ctx:
            self.lib.gcr_context_destroy(self.ctx)
            self.ctx = None


def find_batch_learned(kind, correspondences, sizes, params, proposal, seeds=None, K=None,
                       lo_precision=_abi.GCR_LO_FP64):
    """`find_batch` with the learned order driving PROSAC (params.sampler is
    set to 1). Same arguments and returns as pygcransac.find_batch, plus the
    trained `proposal` and the local optimisation's arithmetic
    (`lo_precision`, GCR_LO_FP64 or GCR_LO_FP32)."""
    torch = _torch()
    lens = [len(c) for c in correspondences]
    offsets = np.zeros(len(lens) + 1, np.int64)
    offsets[1:] = np.cumsum(lens)
    d_corr = torch.from_numpy(np.ascontiguousarray(np.concatenate(correspondences, 0), np.float64)).to(
        proposal.device)
    b = LearnedBatch(proposal, kind, d_corr, offsets, sizes, params, seeds, K, lo_precision=lo_precision)
    try:
        b.prepare()
        b.launch()
        torch.cuda.synchronize()
        return b.results()
    finally:
        b.close()
