"""Brute-force restatement of the seeding semantics for tiny references.

No FM index: every match is found by plain substring search in the text, and
SA-row order is the lexicographic order of the text's suffixes (with the
terminator smallest).  It pins the oracle's definitions independently of the
BWT arithmetic:

* forward candidate e (seed_gen.cu:2127-2265): the 13-mer ending at e must be
  ACGT and occur; the match then grows leftwards while the grown string occurs;
  a non-ACGT base either stops it or is skipped (wildcard), see oracle.h;
* reverse candidate s (seed_gen.cu:2267-2409): the same over the complement
  codes, growing rightwards, searching the string read right to left;
* SMEM / MEM filters, ordering and nested-interval exclusion as in
  seed_gen.cu:991-1139, :927-989, :624-667, :3566-3571.
"""
from __future__ import annotations

ACGT = "ACGT"
FWD_TABLE = 0x24031005
COMP_TABLE = 0x14002035


def encode(read: bytes):
    fwd = [(FWD_TABLE >> ((b & 7) << 2)) & 15 for b in read]
    comp = [(COMP_TABLE >> ((b & 7) << 2)) & 15 for b in read]
    return fwd, comp


def occurrences(text: str, pat: str):
    out, i = [], text.find(pat)
    while i >= 0:
        out.append(i)
        i = text.find(pat, i + 1)
    return out


def rows_order(text: str, positions):
    return sorted(positions, key=lambda p: text[p:])


def seed_read(text: str, read: bytes, k: int, smem: bool, n_stop: bool):
    """Returns [(x, y, positions_in_row_order)] in output order."""
    L = len(read)
    if L < k:
        return []
    F, Cc = encode(read)
    fwd = []  # (x, y, pattern) ascending e
    for e in range(k - 1, L):
        kmer = F[e - 12:e + 1]
        if any(c > 3 for c in kmer):
            continue
        pat = "".join(ACGT[c] for c in kmer)
        if text.find(pat) < 0:
            continue
        b = e - 12
        for i in range(e - 13, -1, -1):
            c = F[i]
            if c > 3:
                if n_stop:
                    break
                b = i
                continue
            cand = ACGT[c] + pat
            if text.find(cand) < 0:
                break
            pat, b = cand, i
        if e - b + 1 >= k:
            fwd.append((b, e + 1, pat))
    rev = []  # ascending s
    for s in range(0, L - k + 1):
        kmer = Cc[s:s + 13]
        if any(c > 3 for c in kmer):
            continue
        pat = "".join(ACGT[c] for c in reversed(kmer))
        if text.find(pat) < 0:
            continue
        x = s + 12
        for i in range(s + 13, L):
            c = Cc[i]
            if c > 3:
                if n_stop:
                    break
                x = i
                continue
            cand = ACGT[c] + pat
            if text.find(cand) < 0:
                break
            pat, x = cand, i
        if x + 1 - s >= k:
            rev.append((s | 0x80000000, (x + 1) | 0x80000000, pat))

    def cnt(p):
        return len(occurrences(text, p)) if p is not None else 0

    nf, nr = len(fwd), len(rev)
    fpat = [r[2] for r in fwd]
    rpat = [r[2] for r in rev]
    if smem:
        for o in range(nf - 1):
            if fwd[o + 1][0] == fwd[o][0]:
                fpat[o] = None
        for o in range(nr - 1, 0, -1):
            if rev[o][1] == rev[o - 1][1]:
                rpat[o] = None
    else:
        keepf = [not (o + 1 < nf and fwd[o + 1][0] == fwd[o][0] and cnt(fwd[o + 1][2]) == cnt(fwd[o][2]))
                 for o in range(nf)]
        keepr = [not (o > 0 and rev[o][1] == rev[o - 1][1] and cnt(rev[o][2]) == cnt(rev[o - 1][2]))
                 for o in range(nr)]
        fpat = [p if kp else None for p, kp in zip(fpat, keepf)]
        rpat = [p if kp else None for p, kp in zip(rpat, keepr)]
    out = []
    a = b = 0
    while a < nf or b < nr:
        if a >= nf:
            take_f = False
        elif b >= nr:
            take_f = True
        else:
            take_f = (fwd[a][0] & 0x7FFFFFFF) <= (rev[b][0] & 0x7FFFFFFF)
        if take_f:
            x, y, _ = fwd[a]
            pat = fpat[a]
            nxt = None
            if pat is not None and not smem:
                for q in range(a + 1, nf):
                    if fwd[q][0] != x:
                        break
                    if fpat[q] is not None:
                        nxt = fpat[q]
                        break
            a += 1
        else:
            x, y, _ = rev[b]
            pat = rpat[b]
            nxt = None
            if pat is not None and not smem:
                for q in range(b - 1, -1, -1):
                    if rev[q][1] != y:
                        break
                    if rpat[q] is not None:
                        nxt = rpat[q]
                        break
            b += 1
        if pat is None:
            continue
        occ = occurrences(text, pat)
        if nxt is not None:
            excl = set(occurrences(text, nxt))
            occ = [p for p in occ if p not in excl]
        if occ:
            out.append((x, y, rows_order(text, occ)))
    return out
