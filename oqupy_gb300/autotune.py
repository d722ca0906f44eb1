"""Launch-shape autotuners for the batched TEMPO kernel.

The bond splits of one instance run on one CTA, so the free parameters are
the CTA width, how many CTAs share an SM and how much shared memory each gets
for working matrices (matrices that do not fit stay in global memory behind
L1/L2).  The best choice depends on the bond dimensions, which grow over a
trajectory: while they are small the batch is throughput-bound (many narrow
CTAs win); once they are large the step is bound by the few largest
instances' split latency (one wide CTA per SM wins).

* ``BucketTuner`` (used on the product path by ``bench.py``): the shape is
  chosen per bond bucket of the running batch.  The first chunk of steps
  spent in a new bucket alternates the candidate shapes launch by launch
  (every tuning launch is a real step of the run), and the faster shape
  serves the rest of the bucket.
* ``tune``: times each candidate shape on a sample of the batch for a few
  steps from the start and returns the fastest; results can be cached per
  (D, dkmax bucket) in a JSON file.
"""

import json
import os
import time
from typing import Dict, List, Optional, Sequence, Tuple

from .tempo import TempoBatch

# (threads per CTA, CTAs per SM, dynamic smem KiB)
CANDIDATES: List[Tuple[int, int, int]] = [
    (256, 3, 56), (256, 2, 88), (256, 1, 200), (192, 3, 56), (128, 4, 48)]


# (threads per CTA, dynamic smem KiB): narrow CTAs, three per SM / one wide CTA per SM
BUCKET_CANDIDATES: List[Tuple[int, int]] = [(512, 200), (256, 56)]


class BucketTuner:
    """Launch shape per bond bucket (``bucket_width`` bond values each).

    ``shape_for(step_in_chunk)`` gives the shape of a launch in the current
    chunk: in the first chunk of an untuned bucket the first ``trials``
    launches per candidate alternate the candidates and the rest of the chunk
    uses the first candidate; ``end_chunk(times)`` takes the chunk's
    per-launch event times and settles the bucket (mean time per shape over
    the interleaved trial launches); ``begin_chunk(max_bond)`` selects the
    bucket of the next chunk.  Pure policy: the caller applies shapes
    (``TempoBatch.set_launch``) and times launches."""

    def __init__(self, candidates: Sequence[Tuple[int, int]] = BUCKET_CANDIDATES,
                 bucket_width: int = 8, trials: int = 2):
        self.candidates = list(candidates)
        self.width = int(bucket_width)
        self.n_trial = max(1, int(trials)) * len(self.candidates)
        self.best: Dict[int, Tuple[int, int]] = {}
        self.trials: Dict[int, Dict[Tuple[int, int], float]] = {}
        self.bucket = 0

    def begin_chunk(self, max_bond: int):
        self.bucket = int(max_bond) // self.width

    def tuning(self) -> bool:
        return self.bucket not in self.best

    def shape_for(self, k: int) -> Tuple[int, int]:
        if self.tuning():
            return self.candidates[k % len(self.candidates)] if k < self.n_trial else self.candidates[0]
        return self.best[self.bucket]

    def end_chunk(self, times_ms: Sequence[float]):
        if not self.tuning() or not times_ms:
            return
        acc: Dict[Tuple[int, int], List[float]] = {}
        for k, t in enumerate(list(times_ms)[: self.n_trial]):
            acc.setdefault(self.shape_for(k), []).append(float(t))
        means = {c: sum(v) / len(v) for c, v in acc.items()}
        self.trials[self.bucket] = means
        self.best[self.bucket] = min(means, key=means.get)

    def table(self) -> Dict[str, List[int]]:
        return {f"bond {b * self.width}-{b * self.width + self.width - 1}": list(c)
                for b, c in sorted(self.best.items())}


def _sm_count() -> int:
    try:
        import torch
        return torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        return 152


def bucket(instances: Sequence[Dict]) -> str:
    D = max(int(i["hs_dim"]) ** 2 for i in instances)
    dk = max(int(i["dkmax"]) if i.get("dkmax") is not None else 10 ** 6 for i in instances)
    return f"D{D}-dk{min(dk, 1000) // 50 * 50}"


def tune(instances: Sequence[Dict], precision: str = "mixed", steps: int = 12,
         sample: int = 0, candidates: Optional[Sequence[Tuple[int, int, int]]] = None,
         cache: Optional[str] = None) -> Dict:
    """Return ``{"block", "ctas_per_sm", "smem_kb", "timings"}`` for the
    fastest candidate on ``instances`` (or a sample of them)."""
    key = f"{precision}:{bucket(instances)}"
    if cache and os.path.exists(cache):
        table = json.load(open(cache))
        if key in table:
            return table[key]
    cands = list(candidates or CANDIDATES)
    insts = list(instances)
    if sample and sample < len(insts):
        stride = len(insts) / sample
        insts = [insts[int(k * stride)] for k in range(sample)]
    sms = _sm_count()
    timings = []
    for block, per_sm, smem in cands:
        b = TempoBatch(insts, precision=precision, out_cap=2, block=block, smem_kb=smem,
                       grid=min(len(insts), per_sm * sms))
        t0 = time.perf_counter()
        b.advance(steps)
        b.info(0)                      # synchronises
        dt = time.perf_counter() - t0
        b.check_status()
        b.close()
        timings.append(((block, per_sm, smem), dt))
    (block, per_sm, smem), _ = min(timings, key=lambda x: x[1])
    res = {"block": block, "ctas_per_sm": per_sm, "smem_kb": smem,
           "timings": [[list(c), t] for c, t in timings]}
    if cache:
        table = json.load(open(cache)) if os.path.exists(cache) else {}
        table[key] = res
        with open(cache, "w") as f:
            json.dump(table, f, indent=1)
    return res
