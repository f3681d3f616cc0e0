"""Box sharding of a level across ranks (one GPU per rank) and the halo exchange between them.

The stage shards by box, as the reference's MPI decomposition does: boxes are independent
within each phase, and the phases are joined by halo exchanges -- the state's ghost cells
before the stage, the ghost faces of utrans and umac (width 1) after MakeUtrans and VelPred
(Source/MaestroMakeUtrans.cpp:631-647, Source/MaestroFill3dData.cpp:425-461), i.e. AMReX's
MultiFab::FillBoundary across ranks.  This module holds the host side of that:

* `sfc_partition`: boxes ordered along a Morton (Z-order) curve of their centres and cut
  into contiguous runs of about equal cell count, as AMReX's space-filling-curve
  DistributionMapping does;
* `halo_plan`: for every box, the pieces of its ghost region that other boxes' valid
  regions cover (periodic images included), split into same-rank copies and one message
  per (sender, receiver) pair;
* `exchange`: the copies and the point-to-point messages (torch.distributed isend / irecv:
  gloo with host tensors, NCCL with device tensors), no collective on the data path, and no
  remote reads -- every piece lands in the receiver's own memory.

A FAB here is a tensor [ncomp, nz, ny, nx] over the valid box grown by the ghost width
(nodal in direction `nodal` for face data), the layout of the library's MultiFabs.
"""
import numpy as np


def _morton(ix, iy, iz, bits=21):
    key = 0
    for b in range(bits):
        key |= ((ix >> b) & 1) << (3 * b) | ((iy >> b) & 1) << (3 * b + 1) | ((iz >> b) & 1) << (3 * b + 2)
    return key


def sfc_partition(boxes, nranks):
    """Owner rank of every box (list of (lo0, lo1, lo2, hi0, hi1, hi2)): boxes in Morton order
    of their centres, cut into nranks contiguous runs whose cell counts are as even as the
    box sizes allow (each cut where the running count first reaches k/nranks of the total)."""
    n = len(boxes)
    if nranks < 1:
        raise ValueError("nranks >= 1")
    cells = [(b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in boxes]
    order = sorted(range(n), key=lambda i: (_morton((boxes[i][0] + boxes[i][3]) // 2 + (1 << 20),
                                                    (boxes[i][1] + boxes[i][4]) // 2 + (1 << 20),
                                                    (boxes[i][2] + boxes[i][5]) // 2 + (1 << 20)), i))
    total = float(sum(cells))
    owner = [0] * n
    run = 0.0
    for i in order:
        r = min(nranks - 1, int(run * nranks / total)) if total > 0 else 0
        owner[i] = r
        run += cells[i]
    return owner


def _valid(b, nodal):
    lo, hi = list(b[:3]), list(b[3:])
    if nodal >= 0:
        hi[nodal] += 1
    return lo, hi


def _intersect(alo, ahi, blo, bhi):
    lo = [max(a, b) for a, b in zip(alo, blo)]
    hi = [min(a, b) for a, b in zip(ahi, bhi)]
    return (lo, hi) if all(l <= h for l, h in zip(lo, hi)) else None


def _subtract(lo, hi, cut_lo, cut_hi):
    """The box [lo, hi] minus [cut_lo, cut_hi], as disjoint boxes."""
    c = _intersect(lo, hi, cut_lo, cut_hi)
    if c is None:
        return [(list(lo), list(hi))]
    out = []
    lo, hi = list(lo), list(hi)
    for d in range(3):
        if lo[d] < c[0][d]:
            a, b = list(lo), list(hi)
            b[d] = c[0][d] - 1
            out.append((a, b))
            lo[d] = c[0][d]
        if hi[d] > c[1][d]:
            a, b = list(lo), list(hi)
            a[d] = c[1][d] + 1
            out.append((a, b))
            hi[d] = c[1][d]
    return out


class HaloPlan:
    """Pieces (dst box, src box, lo, hi in the dst index space, periodic shift) that fill the
    ghost regions of every box from the valid regions of the others.  Each ghost point is
    filled once: where the valid regions of several boxes (or images) cover it -- shared
    nodal faces -- the first in (shift, box) order wins, the same on every rank."""

    def __init__(self, boxes, owner, ng, domain_lo, domain_hi, periodic, nodal=-1):
        self.boxes, self.owner, self.ng, self.nodal = [tuple(b) for b in boxes], list(owner), ng, nodal
        n = [domain_hi[d] - domain_lo[d] + 1 for d in range(3)]
        shifts = [(0, 0, 0)]
        for sx in ((-1, 0, 1) if periodic[0] else (0,)):
            for sy in ((-1, 0, 1) if periodic[1] else (0,)):
                for sz in ((-1, 0, 1) if periodic[2] else (0,)):
                    if (sx, sy, sz) != (0, 0, 0):
                        shifts.append((sx * n[0], sy * n[1], sz * n[2]))
        self.pieces = []
        for dst, bd in enumerate(self.boxes):
            vlo, vhi = _valid(bd, nodal)
            glo, ghi = [v - ng for v in vlo], [v + ng for v in vhi]
            todo = _subtract(glo, ghi, vlo, vhi)
            for sh in shifts:
                for src, bs in enumerate(self.boxes):
                    if src == dst and sh == (0, 0, 0):
                        continue
                    slo, shi = _valid(bs, nodal)
                    slo = [a + s for a, s in zip(slo, sh)]
                    shi = [a + s for a, s in zip(shi, sh)]
                    rest = []
                    for lo, hi in todo:
                        c = _intersect(lo, hi, slo, shi)
                        if c is None:
                            rest.append((lo, hi))
                            continue
                        self.pieces.append((dst, src, c[0], c[1], sh))
                        rest += _subtract(lo, hi, c[0], c[1])
                    todo = rest

    def messages(self):
        """{(sender, receiver): [piece indices]} of the pieces whose boxes are on two ranks,
        in plan order (both sides see the same list)."""
        m = {}
        for q, (dst, src, lo, hi, sh) in enumerate(self.pieces):
            a, b = self.owner[src], self.owner[dst]
            if a != b:
                m.setdefault((a, b), []).append(q)
        return m

    def cells_sent(self):
        """Ghost points that cross ranks, per exchange (the halo volume of the partition)."""
        tot = 0
        for q in [q for v in self.messages().values() for q in v]:
            _, _, lo, hi, _ = self.pieces[q]
            tot += int(np.prod([h - l + 1 for l, h in zip(lo, hi)]))
        return tot


def _view(fab, box, nodal, ng, lo, hi):
    """Slice of a FAB tensor [nc, nz, ny, nx] (valid box `box` grown by ng) over [lo, hi]."""
    vlo, _ = _valid(box, nodal)
    flo = [v - ng for v in vlo]
    return fab[:, lo[2] - flo[2]:hi[2] - flo[2] + 1, lo[1] - flo[1]:hi[1] - flo[1] + 1,
               lo[0] - flo[0]:hi[0] - flo[0] + 1]


def exchange(plan, fabs, rank, dist=None):
    """FillBoundary of a sharded MultiFab: fabs maps every box this rank owns to its FAB.
    Same-rank pieces are copied; the others travel as one message per (sender, receiver)
    pair, packed in plan order, by point-to-point isend / irecv (no collective)."""
    import torch
    ng, nodal = plan.ng, plan.nodal

    def src_piece(q):
        dst, src, lo, hi, sh = plan.pieces[q]
        return _view(fabs[src], plan.boxes[src], nodal, ng, [a - s for a, s in zip(lo, sh)],
                     [a - s for a, s in zip(hi, sh)])

    def dst_piece(q):
        dst, src, lo, hi, sh = plan.pieces[q]
        return _view(fabs[dst], plan.boxes[dst], nodal, ng, lo, hi)

    msgs = plan.messages()
    reqs, inbox = [], []
    if dist is not None:
        for (a, b), qs in sorted(msgs.items()):
            if a == rank:
                buf = torch.cat([src_piece(q).reshape(-1) for q in qs]).contiguous()
                reqs.append(dist.isend(buf, dst=b))
                inbox.append(buf)  # kept alive until the send completes
            elif b == rank:
                size = sum(int(np.prod(dst_piece(q).shape)) for q in qs)
                buf = torch.empty(size, dtype=fabs[plan_first_owned(plan, rank)].dtype,
                                  device=fabs[plan_first_owned(plan, rank)].device)
                reqs.append(dist.irecv(buf, src=a))
                inbox.append((qs, buf))
    for q, (dst, src, lo, hi, sh) in enumerate(plan.pieces):
        if plan.owner[dst] == rank and plan.owner[src] == rank:
            dst_piece(q).copy_(src_piece(q))
    for r in reqs:
        r.wait()
    for item in inbox:
        if isinstance(item, tuple):
            qs, buf = item
            off = 0
            for q in qs:
                v = dst_piece(q)
                n = int(np.prod(v.shape))
                v.copy_(buf[off:off + n].reshape(v.shape))
                off += n


def plan_first_owned(plan, rank):
    for b, o in enumerate(plan.owner):
        if o == rank:
            return b
    raise ValueError(f"rank {rank} owns no box")
