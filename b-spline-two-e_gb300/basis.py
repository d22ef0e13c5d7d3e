"""Symmetry blocks of the two-electron basis (src/tools/orbital_tools.f90:245-343).

symmetries() lists (L, M, parity) in the order init_basis creates them; the
configuration list of each block comes from the library (bs2e_configs, a
restatement of count_configs).  spin = 1 adds the triplet blocks, which the
reference does not build.
"""


def count_terms(max_L, z_pol, two_el=True):
    """count_terms (orbital_tools.f90:245-261)."""
    if z_pol:
        return max_L + 1
    if two_el:
        return (max_L + 1) ** 2
    return max_L + 1 + max_L * (max_L + 1) // 2


def symmetries(max_L, z_pol=True, two_el=True):
    """(L, M, parity_odd) of every block in init_basis order (orbital_tools.f90:285-342)."""
    out = [(0, 0, 0)]
    if z_pol:
        for L in range(1, max_L + 1):
            out.append((L, 0, L % 2))
    else:
        for L in range(1, max_L + 1):
            if two_el:
                for p in (0, 1):
                    for M in range(-L, L + 1):
                        if abs(M % 2) != p:
                            continue
                        out.append((L, M, p))
            else:
                for M in range(-L, L + 1, 2):
                    out.append((L, M, L % 2))
    assert len(out) == count_terms(max_L, z_pol, two_el)
    return out


def block_work(n_config, n_channels):
    """Relative assembly work of a block: rows times column channels."""
    return int(n_config) * max(int(n_channels), 1)


def shard_blocks(work, world_size, rank):
    """Indices of the symmetry blocks rank `rank` assembles.

    Blocks are independent (no data exchange between them), so a multi-GPU
    basis setup hands each rank whole blocks: greedy longest-first assignment
    to the least loaded rank, ties broken by block index so every rank
    computes the same partition without communicating.
    """
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    load = [0] * world_size
    owner = [0] * len(work)
    for i in order:
        r = min(range(world_size), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += work[i]
    return [i for i in range(len(work)) if owner[i] == rank]
