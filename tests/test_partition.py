"""Box sharding across ranks (maestroex_gb300/partition.py): the space-filling-curve
partition, the halo plan, and the exchange of ghost cells and ghost faces between ranks by
point-to-point messages -- checked against the domain-wide fill on one rank, and with two
and three gloo processes on the CPU."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from maestroex_gb300 import configs  # noqa: E402
from maestroex_gb300.partition import HaloPlan, exchange, sfc_partition  # noqa: E402

N = (24, 16, 20)
PERIODIC = (True, True, False)


def layout():
    return configs.uneven_boxes(N, [4, 8], np.random.default_rng(3))


def domain_field(nc, nodal, seed=5):
    """Seeded data; face data in a periodic direction has its two copies of the periodic face
    equal, as a MAC velocity does (otherwise which copy a ghost takes is not defined)."""
    n = list(N)
    if nodal >= 0:
        n[nodal] += 1
    f = np.random.default_rng(seed).standard_normal((nc, n[2], n[1], n[0]))
    if nodal >= 0 and PERIODIC[nodal]:
        ax = 3 - nodal
        idx = [slice(None)] * 4
        src = list(idx)
        idx[ax], src[ax] = N[nodal], 0
        f[tuple(idx)] = f[tuple(src)]
    return f


def fabs_of(boxes, field, ng, nodal, owned):
    """Every owned box's FAB: valid points from the domain field, ghosts NaN."""
    out = {}
    for b, bx in enumerate(boxes):
        if b not in owned:
            continue
        lo, hi = list(bx[:3]), list(bx[3:])
        if nodal >= 0:
            hi[nodal] += 1
        f = np.full((field.shape[0],) + tuple(hi[d] - lo[d] + 1 + 2 * ng for d in (2, 1, 0)), np.nan)
        f[:, ng:-ng, ng:-ng, ng:-ng] = field[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
        out[b] = torch.from_numpy(f)
    return out


def expected_fab(bx, field, ng, nodal):
    """The FAB FillBoundary leaves: domain values, periodic images wrapped; ghost points
    outside a non-periodic face stay NaN (the physical-boundary fill is another step)."""
    nc = field.shape[0]
    lo, hi = list(bx[:3]), list(bx[3:])
    if nodal >= 0:
        hi[nodal] += 1
    f = np.full((nc,) + tuple(hi[d] - lo[d] + 1 + 2 * ng for d in (2, 1, 0)), np.nan)
    n = [N[d] + (1 if d == nodal else 0) for d in range(3)]
    per = [N[d] for d in range(3)]
    for k in range(lo[2] - ng, hi[2] + ng + 1):
        for j in range(lo[1] - ng, hi[1] + ng + 1):
            for i in range(lo[0] - ng, hi[0] + ng + 1):
                p = [i, j, k]
                ok = True
                for d in range(3):
                    if p[d] < 0 or p[d] >= n[d]:
                        if PERIODIC[d]:
                            p[d] %= per[d]
                        else:
                            ok = False
                if ok:
                    f[:, k - lo[2] + ng, j - lo[1] + ng, i - lo[0] + ng] = field[:, p[2], p[1], p[0]]
    return f


def test_sfc_partition_is_balanced_and_contiguous():
    boxes = layout()
    cells = np.array([(b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in boxes])
    for nranks in (1, 2, 3, 5):
        owner = np.array(sfc_partition(boxes, nranks))
        assert set(owner) == set(range(nranks))
        per = np.array([cells[owner == r].sum() for r in range(nranks)])
        assert per.max() - per.min() <= 2 * cells.max()


@pytest.mark.parametrize("nodal,ng", [(-1, 3), (-1, 4), (2, 1), (0, 1)])
def test_halo_plan_on_one_rank_is_fill_boundary(nodal, ng):
    boxes = layout()
    owner = [0] * len(boxes)
    plan = HaloPlan(boxes, owner, ng, (0, 0, 0), tuple(n - 1 for n in N), PERIODIC, nodal)
    field = domain_field(2, nodal)
    fabs = fabs_of(boxes, field, ng, nodal, set(range(len(boxes))))
    exchange(plan, fabs, 0)
    for b, bx in enumerate(boxes):
        assert np.array_equal(fabs[b].numpy(), expected_fab(bx, field, ng, nodal), equal_nan=True), b


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, nodal, ng, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    boxes = layout()
    owner = sfc_partition(boxes, ws)
    plan = HaloPlan(boxes, owner, ng, (0, 0, 0), tuple(n - 1 for n in N), PERIODIC, nodal)
    field = domain_field(3, nodal, seed=11)
    mine = {b for b, o in enumerate(owner) if o == rank}
    fabs = fabs_of(boxes, field, ng, nodal, mine)
    exchange(plan, fabs, rank, dist)
    bad = [b for b in mine if not np.array_equal(fabs[b].numpy(), expected_fab(boxes[b], field, ng, nodal),
                                                 equal_nan=True)]
    out[rank] = (len(mine), bad, plan.cells_sent())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("ws,nodal,ng", [(2, -1, 3), (3, -1, 4), (2, 2, 1), (3, 1, 1)])
def test_exchange_across_gloo_ranks(ws, nodal, ng):
    """Each rank holds only its boxes; after the exchange every ghost point a neighbour's
    valid region covers (periodic images included) holds the domain's value."""
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, _free_port(), nodal, ng, out), nprocs=ws, join=True)
        res = dict(out)
    assert sum(r[0] for r in res.values()) == len(layout())
    for r in range(ws):
        assert res[r][1] == [], f"rank {r}: boxes with wrong ghosts {res[r][1]}"
        assert res[r][2] > 0  # the partition does cut: ghost points cross ranks
