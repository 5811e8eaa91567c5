"""Members of a batched ensemble split across ranks (one GPU per rank).

The members are independent basins, so a multi-GPU ensemble needs no data
exchange: each rank steps its own share, and only the per-member results
(integrals) are gathered on the host.  Shares are balanced by cell count,
since a member's step time grows with its cells: members are taken
largest first and each goes to the rank with the fewest cells so far (ties
to the lower rank), which bounds the imbalance by one member's cells.
"""


def partition_members(cells, nranks):
    """List, per rank, of the member indices (ascending) it steps, for
    members of the given cell counts."""
    if nranks < 1:
        raise ValueError('nranks must be at least 1')
    load = [0] * nranks
    share = [[] for _ in range(nranks)]
    for i in sorted(range(len(cells)), key=lambda k: (-cells[k], k)):
        r = min(range(nranks), key=lambda q: (load[q], q))
        share[r].append(i)
        load[r] += cells[i]
    return [sorted(s) for s in share]


def member_cells(case):
    """Cells of one member, (Nx - 1)(Ny - 1), the unit of the metric."""
    return (case['config']['nx'] - 1) * (case['config']['ny'] - 1)
