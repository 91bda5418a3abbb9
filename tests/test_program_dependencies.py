"""The generated recursion program (codegen.program_data) is race-free and
complete: walking its stages with the index arithmetic of the kernel's item
types (mf_me_rec.cuh: rec_current, rec_item, rec_st_A), every value an item
reads was written by an earlier stage (or is an external wavefunction),
no two items of a stage write the same slot, every index is in range, and
the amplitude stage finds everything it reads."""
import pytest

from madflow_gb300 import codegen


def _bitrev(x, n):
    return sum(((x >> j) & 1) << (n - 1 - j) for j in range(n))


def _item_access(d, typ, L, r, sub):
    """(reads, writes) of one item as sets of (array, index)."""
    prog, k = d["prog"], d["k"]
    reads, writes = set(), set()

    def current_reads(Lc):
        for i in range(1, Lc):
            ja, jb = prog[r + 4 * i], prog[r + 4 * i + 1]
            reads.add(("J", ja + (sub & ((1 << i) - 1))))
            reads.add(("J", jb + (sub >> i)))
        q = r + 4 * Lc
        for i in range(1, Lc):
            for j in range(i + 1, Lc):
                x, y, z = prog[q], prog[q + 1], prog[q + 2]
                reads.add(("J", x + (sub & ((1 << i) - 1))))
                reads.add(("J", y + ((sub >> i) & ((1 << (j - i)) - 1))))
                reads.add(("J", z + (sub >> j)))
                q += 4

    if typ == 0:
        current_reads(L)
        writes.add(("J", prog[r] + sub))
        writes.add(("J", prog[r + 1] + _bitrev(sub, L)))
    elif typ == 1:
        current_reads(k)
        s, srev = prog[r], prog[r + 1]
        nc = 1 << (k + 2)
        # the helicity index of the amplitude slot is the unpacked pattern
        hg = d["hunpack"][s * (1 << k) + sub]
        for q in range(4):
            c = hg | ((q & 1) << k) | ((q >> 1) << (k + 1))
            writes.add(("A", s * nc + c))
            writes.add(("A", srev * nc + c))
    elif typ == 2:
        ht, hp = sub >> L, sub & ((1 << L) - 1)
        for i in range(L):
            prev, jsuf = prog[r + 2 + 2 * i], prog[r + 3 + 2 * i]
            reads.add(("J", jsuf + (hp >> i)))
            if prev >= 0:
                reads.add(("O", prev + (ht << i) + (hp & ((1 << i) - 1))))
        writes.add(("O", prog[r] + sub))
    elif typ == 3:
        hp = sub & ((1 << L) - 1)
        reads.add(("J", prog[r + 1] + hp))
        writes.add(("RW", prog[r] + sub))
    elif typ == 4:
        o = prog[r] + sub
        reads.add(("O", o))
        writes.add(("MP", 2 * o))
        writes.add(("MP", 2 * o + 1))
    else:
        raise AssertionError(f"unknown item type {typ}")
    return reads, writes


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_program_is_race_free_and_complete(k):
    d = codegen.program_data(k)
    size = {"J": d["J_TOTAL"], "O": d["O_TOTAL"], "RW": d["R_TOTAL"], "MP": 8 * k,
            "A": len(codegen.permutations(k)) << (k + 2)}
    ready = {("J", d["jo_ext"][q] + h) for q in range(k) for h in range(2)}
    pdesc, first = d["pdesc"], d["stage_first"]
    for st in range(1, k):
        stage_writes = set()
        for part in range(first[st - 1], first[st]):
            typ, L, nodes, rec0, rsz = pdesc[5 * part: 5 * part + 5]
            lper = L if typ <= 1 else L + 1
            for n in range(nodes):
                for sub in range(1 << lper):
                    reads, writes = _item_access(d, typ, L, rec0 + n * rsz, sub)
                    for a, i in reads | writes:
                        assert 0 <= i < size[a], (k, st, typ, a, i)
                    missing = reads - ready
                    assert not missing, (k, st, typ, sorted(missing)[:4])
                    clash = writes & stage_writes
                    assert not clash, (k, st, typ, sorted(clash)[:4])
                    stage_writes |= writes
        ready |= stage_writes
    # every amplitude slot is written once the last stage is done
    assert {("A", i) for i in range(size["A"])} <= ready
    # the amplitude stage
    nperm = len(codegen.permutations(k))
    arec = d["arec"]
    for s in range(nperm):
        for hfull in range(1 << k):
            for i in range(1, k):
                oo, ro = arec[s * 2 * (k - 1) + 2 * (i - 1)], arec[s * 2 * (k - 1) + 2 * (i - 1) + 1]
                lo, hi = hfull & ((1 << i) - 1), hfull >> i
                if d["use_mp"] and i == 1:
                    need = {("J", ro + hi)} | {("MP", 2 * (oo + (ht << 1) + lo) + tb) for ht in (0, 1) for tb in (0, 1)}
                else:
                    need = {("O", oo + lo), ("O", oo + (1 << i) + lo), ("RW", ro + hi),
                            ("RW", ro + (1 << (k - i)) + hi)}
                assert need <= ready, (k, s, i, sorted(need - ready)[:4])
