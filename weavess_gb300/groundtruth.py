"""Exact k-NN ground truth for recall@k, on the GPU.

Candidates come from an FP32 brute force (torch matmul in FP32, no TF32),
then a margin of candidates is re-ranked with FP64 distances in the direct
form sum((q - x)^2); ties break by smaller id.  For integer-valued data in
[0, 255] at d <= 128 the FP32 pass is already exact (every partial sum is an
integer below 2^24).  This is measurement code (the recall judge), not part of
the searched path.
"""
from __future__ import annotations

import numpy as np


def knn_fp64(base: np.ndarray, query: np.ndarray, k: int = 100, margin: int = 64, device="cuda",
             q_chunk: int = 1024, b_chunk: int = 1 << 20) -> np.ndarray:
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        B = torch.from_numpy(np.ascontiguousarray(base, np.float32)).to(device)
        bn = (B.double() ** 2).sum(1).float()
        kk = min(k + margin, B.shape[0])
        out = np.empty((query.shape[0], k), np.uint32)
        for s in range(0, query.shape[0], q_chunk):
            Q = torch.from_numpy(np.ascontiguousarray(query[s:s + q_chunk], np.float32)).to(device)
            qn = (Q.double() ** 2).sum(1).float()
            best_d = best_i = None
            for b0 in range(0, B.shape[0], b_chunk):
                Bc = B[b0:b0 + b_chunk]
                d = qn[:, None] + bn[None, b0:b0 + b_chunk] - 2.0 * (Q @ Bc.T)
                dv, di = torch.topk(d, min(kk, Bc.shape[0]), dim=1, largest=False)
                di = di + b0
                if best_d is None:
                    best_d, best_i = dv, di
                else:
                    cd = torch.cat([best_d, dv], 1)
                    ci = torch.cat([best_i, di], 1)
                    best_d, o = torch.topk(cd, kk, dim=1, largest=False)
                    best_i = torch.gather(ci, 1, o)
            # FP64 rerank of the candidates, ties by id
            cand = B[best_i].double()
            dd = ((cand - Q.double()[:, None, :]) ** 2).sum(2)
            ids = best_i.cpu().numpy()
            dnp = dd.cpu().numpy()
            for r in range(ids.shape[0]):
                o = np.lexsort((ids[r], dnp[r]))[:k]
                out[s + r] = ids[r, o]
        return out
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
