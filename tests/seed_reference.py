"""Record-by-record restatement of overlap_read (src/overlap.F90:234-366) and of the .eig
reader (src/readwrite.F90:583-635): the checker for the parallel native readers.  Each
READ takes the leading items of one non-blank record; Fortran 'd' exponents are read."""
import numpy as np


def _records(path):
    lines = open(path).read().split("\n")
    head, rest = lines[:2], [l for l in lines[2:] if l.replace(",", " ").strip()]
    return head, rest


def _f(x):
    return float(x.replace("d", "e").replace("D", "e"))


def _items(line):
    return line.replace(",", " ").split()


def read_mmn(path, nnlist, nncell):
    head, rec = _records(path)
    nb, nk, nntot = (int(x) for x in _items(head[1])[:3])
    m = np.zeros((nb, nb, nntot, nk), dtype=np.complex128, order="F")
    r = 0
    for _ in range(nk * nntot):
        h = [int(x) for x in _items(rec[r])[:5]]
        r += 1
        blk = np.zeros(nb * nb, dtype=np.complex128)
        for i in range(nb * nb):
            it = _items(rec[r])
            blk[i] = _f(it[0]) + 1j * _f(it[1])
            r += 1
        k, k2 = h[0] - 1, h[1] - 1
        hit = [b for b in range(nntot) if nnlist[k][b] == k2 and tuple(nncell[k][b]) == tuple(h[2:5])]
        if len(hit) != 1:
            raise ValueError("neighbour not found / not unique")
        m[:, :, hit[0], k] = blk.reshape(nb, nb, order="F")
    return m


def read_amn(path):
    head, rec = _records(path)
    nb, nk, npj = (int(x) for x in _items(head[1])[:3])
    a = np.zeros((nb, npj, nk), dtype=np.complex128, order="F")
    for r in range(nb * npj * nk):
        it = _items(rec[r])
        a[int(it[0]) - 1, int(it[1]) - 1, int(it[2]) - 1] = _f(it[3]) + 1j * _f(it[4])
    return a


def read_eig(path, nb, nk):
    rec = [l for l in open(path).read().split("\n") if l.strip()]
    e = np.zeros((nb, nk), order="F")
    r = 0
    for k in range(nk):
        for n in range(nb):
            it = _items(rec[r])
            if int(it[0]) != n + 1 or int(it[1]) != k + 1:
                raise ValueError("mismatch")
            e[n, k] = _f(it[2])
            r += 1
    return e
