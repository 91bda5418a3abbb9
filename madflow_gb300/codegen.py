"""Process generator for g g > t t~ + (k-2) g: colour basis, colour matrix,
helicity table, diagram count and the CUDA source of the colour-ordered
amplitude recursion.

This takes the place of madflow's PyOut exporter (madgraph_plugin/
PyOut_exporter.py:125-285, which needs MG5_aMC) for the process family the
benchmarks use.  Instead of a list of Feynman diagrams it emits a Berends-Giele
recursion over colour-ordered currents (Berends & Giele, Nucl. Phys. B306
(1988) 759), in the fundamental-trace colour basis

    M = sum_sigma (T^{a_sigma1} ... T^{a_sigmak})_{i_t j_tbar} A(sigma),
    |M|^2 = sum_{sigma,tau} A(sigma) C_{sigma tau} A(tau)^*,

which is the same basis MadGraph uses for a single quark line (for gg > tt~
the colour matrix is madflow's [[16,-2],[-2,16]]/3, tests/mockup_debug_me.py:506-507).

Vertex normalisation matches the ALOHA routines of the reference with MadGraph's
SM couplings GC_10 = -g_s (ggg), GC_11 = i g_s (ttg), GC_12 = i g_s^2 (gggg):
the colour-ordered three-gluon current carries -i*GC_10 and the four-gluon
current -GC_12 relative to the full-colour vertices.

Particle order is MadGraph's: 0, 1 incoming gluons, 2 = t, 3 = t~, 4.. outgoing
gluons.  Gluon label j (0..k-1) is particle GLUON_PARTICLE[j].
"""
from fractions import Fraction
from functools import lru_cache
import itertools
import math

GLUON_PARTICLE = (0, 1, 4, 5, 6, 7)
NC = 3
KNOWN_DIAGRAMS = {2: 3, 3: 16, 4: 123, 5: 1240}


# ---------------------------------------------------------------------------
# colour algebra: sums over adjoint labels of products of traces of T^a
# (Tr T^a T^b = delta/2), reduced with the Fierz identity
#   sum_a T^a_ij T^a_kl = 1/2 (delta_il delta_kj - 1/N delta_ij delta_kl)
# ---------------------------------------------------------------------------
def _canon(traces):
    """Canonical form of a product of traces up to cyclic rotation and label
    renaming (labels appear exactly twice overall)."""
    best = None
    # rotations of each trace, then order of traces; relabel by first appearance
    rots = []
    for t in traces:
        if not t:
            rots.append([()])
        else:
            rots.append([t[i:] + t[:i] for i in range(len(t))])
    for choice in itertools.product(*rots):
        for order in itertools.permutations(range(len(choice))):
            seq = [choice[i] for i in order]
            mapping = {}
            out = []
            for t in seq:
                nt = []
                for lab in t:
                    if lab not in mapping:
                        mapping[lab] = len(mapping)
                    nt.append(mapping[lab])
                out.append(tuple(nt))
            key = tuple(out)
            if best is None or key < best:
                best = key
    return best


@lru_cache(maxsize=None)
def _trace_sum(traces):
    """Sum over all adjoint labels of prod_i Tr(traces[i]); exact Fraction."""
    traces = [t for t in traces]
    # empty traces give N each
    factor = Fraction(1)
    rest = []
    for t in traces:
        if len(t) == 0:
            factor *= NC
        else:
            rest.append(t)
    if not rest:
        return factor
    # a single generator in a trace vanishes
    for t in rest:
        if len(t) == 1:
            return Fraction(0)
    lab = rest[0][0]
    # locate second occurrence
    for ti, t in enumerate(rest):
        idx = [i for i, x in enumerate(t) if x == lab]
        if ti == 0 and len(idx) == 2:
            i, j = idx
            Y = t[i + 1 : j]
            X = t[j + 1 :] + t[:i]
            others = rest[1:]
            # Tr(T^a Y T^a X) = 1/2 Tr(Y) Tr(X) - 1/(2N) Tr(Y X)
            a = _trace_sum(_canon(others + [Y, X]))
            b = _trace_sum(_canon(others + [Y + X]))
            return factor * (Fraction(1, 2) * a - Fraction(1, 2 * NC) * b)
        if ti > 0 and idx:
            t0 = rest[0]
            j = idx[0]
            # rotate so the label is last in both
            X = t0[1:]
            Y = t[j + 1 :] + t[:j]
            others = [r for q, r in enumerate(rest) if q not in (0, ti)]
            # Tr(X T^a) Tr(Y T^a) = 1/2 Tr(X Y) - 1/(2N) Tr(X) Tr(Y)
            a = _trace_sum(_canon(others + [X + Y]))
            b = _trace_sum(_canon(others + [X, Y]))
            return factor * (Fraction(1, 2) * a - Fraction(1, 2 * NC) * b)
    raise ValueError("label without partner")


def permutations(k):
    """Colour orderings in lexicographic order (the colour-flow index)."""
    return list(itertools.permutations(range(k)))


@lru_cache(maxsize=None)
def colour_matrix(k):
    """Exact colour matrix C[sigma][tau] = sum Tr(T^{s1}..T^{sk} T^{tk}..T^{t1}).

    Returns (numerators, denominator) with integer numerators and the common
    denominator, so that C = numerators / denominator exactly.
    """
    perms = permutations(k)
    index = {p: i for i, p in enumerate(perms)}
    # row of the identity ordering; C[s][t] = C[id][s^-1 t]
    row = []
    ident = tuple(range(k))
    for t in perms:
        word = ident + tuple(reversed(t))
        row.append(_trace_sum(_canon([word])))
    n = len(perms)
    C = [[None] * n for _ in range(n)]
    for si, s in enumerate(perms):
        inv = [0] * k
        for pos, lab in enumerate(s):
            inv[lab] = pos
        for ti, t in enumerate(perms):
            comp = tuple(inv[lab] for lab in t)
            C[si][ti] = row[index[comp]]
    den = 1
    for r in C:
        for v in r:
            den = den * v.denominator // math.gcd(den, v.denominator)
    num = [[int(v * den) for v in r] for r in C]
    return num, den


def helicities(k):
    """Helicity combinations in MadGraph's order (the t~ runs +1 then -1)."""
    n = k + 2
    out = []
    for c in range(1 << n):
        h = []
        for i in range(n):
            bit = (c >> (n - 1 - i)) & 1
            v = 1.0 if bit else -1.0
            if i == 3:
                v = -v
            h.append(v)
        out.append(h)
    return out


def denominator(k):
    """Initial-state average (8*8 colours x 2*2 helicities) times the symmetry
    factor of identical final-state gluons."""
    return 256 * math.factorial(k - 2)


def diagram_count(k):
    """Number of tree Feynman diagrams (ggg, gggg, ttg vertices) with k gluons
    attached to the top line, counted with unordered (colour-dressed) currents."""
    full = (1 << k) - 1
    G = {}
    for s in range(1, full + 1):
        pc = bin(s).count("1")
        if pc == 1:
            G[s] = 1
            continue
        low = s & -s
        tot = 0
        sub = (s - 1) & s
        while sub:
            if sub & low:
                tot += G[sub] * G[s ^ sub]
            sub = (sub - 1) & s
        # three-way splits
        s1 = s
        while s1:
            if (s1 & low) and s1 != s:
                rest = s ^ s1
                low2 = rest & -rest
                s2 = rest
                while s2:
                    if (s2 & low2) and s2 != rest:
                        tot += G[s1] * G[s2] * G[rest ^ s2]
                    s2 = (s2 - 1) & rest
            s1 = (s1 - 1) & s
        G[s] = tot
    O = {0: 1}
    for s in range(1, full):
        tot = 0
        b = s
        while b:
            tot += O[s ^ b] * G[b]
            b = (b - 1) & s
        O[s] = tot
    amp = 0
    b = full
    while b:
        amp += O[full ^ b] * G[b]
        b = (b - 1) & full
    return amp


def process_name(k):
    return "gg_ttx" + "g" * (k - 2)


# ---------------------------------------------------------------------------
# CUDA emission
# ---------------------------------------------------------------------------
def _mask(seq):
    m = 0
    for g in seq:
        m |= 1 << g
    return m


def _canonical(seq):
    """(representative, sign) with J(reverse s) = (-1)^(|s|+1) J(s)."""
    rev = tuple(reversed(seq))
    if seq <= rev:
        return seq, 1
    return rev, (-1) ** (len(seq) + 1)


def colour_tc_operand(k):
    """The colour numerators as the B operand (N x K, K-major, 32-bit) of a
    tensor-core MMA, in the no-swizzle canonical shared-memory layout: core
    matrices of 8 rows x 16 bytes stored contiguously, neighbours along K
    TC_LBO = 128 bytes apart, neighbouring 8-row groups TC_SBO = NPERM/4 x
    128 bytes apart.  N is padded to a multiple of 16 with zero rows.
    B[n][k] = C[k][n].  Returns (padded N, flat list of floats)."""
    num, _ = colour_matrix(k)
    n = len(num)
    if n % 4:
        raise ValueError("the canonical layout needs a multiple of 4 colour flows")
    npad = -(-n // 16) * 16
    lbo, sbo = 32, (n // 4) * 32  # in 4-byte elements
    out = [0.0] * ((npad // 8) * sbo)
    for r in range(npad):
        for c in range(n):
            out[(r // 8) * sbo + (c // 4) * lbo + (r % 8) * 4 + (c % 4)] = float(num[c][r]) if r < n else 0.0
    return npad, out


def emit_process_header(k):
    """Header with the process constants and the amplitude recursion."""
    num, den = colour_matrix(k)
    hels = helicities(k)
    n = len(num)
    L = []
    L.append(f"// Generated by madflow_gb300.codegen: g g > t t~{' g' * (k - 2)} ({diagram_count(k)} diagrams,")
    L.append(f"// {n} colour flows, {len(hels)} helicities).  Do not edit.")
    L.append("#pragma once")
    L.append(f"namespace ttng{k} {{")
    L.append(f"constexpr int K = {k};")
    L.append(f"constexpr int NPERM = {n};")
    L.append(f"constexpr int NCOMB = {len(hels)};")
    L.append(f"constexpr int NEXT = {k + 2};")
    L.append(f"constexpr double DENOMINATOR = {float(denominator(k))!r};")
    L.append(f"constexpr double COLOUR_DEN = {float(den)!r};")
    L.append(f"static __constant__ float colour_num[{n * n}] = {{")
    for r in num:
        L.append("  " + ", ".join(f"{float(v)!r}f" for v in r) + ",")
    L.append("};")
    L.append(f"static __constant__ signed char hel[{len(hels)}][{k + 2}] = {{")
    for h in hels:
        L.append("  {" + ", ".join(str(int(v)) for v in h) + "},")
    L.append("};")
    if n % 4 == 0:
        npad, tcb = colour_tc_operand(k)
        L.append("// the colour numerators as a tensor-core B operand (colour_tc_operand)")
        L.append(f"constexpr int TC_N = {npad};")
        L.append("constexpr int TC_LBO = 128;")
        L.append(f"constexpr int TC_SBO = {(n // 4) * 128};")
        L.append(f"__device__ __align__(16) const float colour_tc_b[{len(tcb)}] = {{")
        for i in range(0, len(tcb), 16):
            L.append("  " + ", ".join(f"{v!r}f" for v in tcb[i:i + 16]) + ",")
        L.append("};")
    L.append("// host copies for the handle's info calls")
    L.append(f"static const float colour_num_h[{n * n}] = {{")
    for r in num:
        L.append("  " + ", ".join(f"{float(v)!r}f" for v in r) + ",")
    L.append("};")
    L.append(f"static const signed char hel_h[{len(hels)}][{k + 2}] = {{")
    for h in hels:
        L.append("  {" + ", ".join(str(int(v)) for v in h) + "},")
    L.append("};")
    L.append("}  // namespace")
    L.append(emit_program(k))
    return "\n".join(L) + "\n"


def _code(seq, base):
    c = 0
    for j, g in enumerate(seq):
        c += (g + 1) * base**j
    return c


def _arr(name, ctype, vals):
    vals = list(vals) or [0]
    body = ", ".join(str(int(v)) for v in vals)
    return f"__device__ const {ctype} {name}[{len(vals)}] = {{{body}}};\nstatic const {ctype} {name}_h[{len(vals)}] = {{{body}}};"


def _bitrev(h, n):
    r = 0
    for j in range(n):
        r |= ((h >> j) & 1) << (n - 1 - j)
    return r


def program_data(k):
    """The helicity-recycling evaluation of mf_me_rec.cuh as a flat program.

    Storage (shared memory of one event):
      J  every ordered gluon sequence s of length 1..k-1, 2^|s| helicity
         patterns (length 1: the external gluons);
      O  every ordered prefix a (gluons next to the top) of length 1..k-1,
         2 x 2^|a| (top helicity, pattern);
      R  every ordered suffix b of length 1..k-1, 2 x 2^|b| (t~ helicity,
         pattern): the row wtb^T S(J(b));
      T0 every ordering sigma, 2^k x 4: wtb^T S(J(sigma)) wt.
    A helicity pattern of a sequence packs the helicity bit of its j-th gluon
    at bit j, so the patterns of the parts of a split are shifts and masks.
    Only one of each pair (s, reverse s) is computed; the other is written
    with J(reverse s; bitrev(h)) = (-1)^(|s|+1) J(s; h).

    Stage L (1 <= L <= k-1) holds the gluon currents of length L+1, the top
    currents of length L, the t~ rows of length L and, at L = k-1, the bare
    full-length contractions T0; every item depends on earlier stages only.

    From four gluons on, the t~ rows of length k-1 are not built: the
    amplitude terms they enter, R(b) . O(a) with |a| = 1, are evaluated as
    J(b) . MP(a), MP(a)^mu = wtb^T S(e_mu) O(a) the bilinears of the 4k
    one-gluon top currents (stage 2, part type 4), which are far fewer than
    the rows.  Their storage is kept (the tensor-core colour operands use
    it).
    """
    seqs = [s for L in range(1, k) for s in itertools.permutations(range(k), L)]
    jo, off = {}, 0
    for s in seqs:
        jo[s] = off
        off += 1 << len(s)
    J_TOTAL = off
    oo, off = {}, 0
    for s in seqs:
        oo[s] = off
        off += 2 << len(s)
    O_TOTAL = off
    ro, off = {}, 0
    for s in seqs:
        ro[s] = off
        off += 2 << len(s)
    R_TOTAL = off
    perms = permutations(k)
    pidx = {p: i for i, p in enumerate(perms)}

    prog = []  # flat int records
    parts = []  # per stage: list of (type, L, n_nodes, first_record, record_size)

    # Records are groups of four ints, so that the kernels read each group
    # with one 16-byte load: a current's header (out, reversed out, sign,
    # subset), one group per split (J offsets and subsets of both sides), one
    # per triple of the contact term (three J offsets, padding).
    def cur_record(s, out_off, out_rev, sign):
        L = len(s)
        rec = [out_off, out_rev, sign, _mask(s)]
        for i in range(1, L):
            a, b = s[:i], s[i:]
            rec += [jo[a], jo[b], _mask(a), _mask(b)]
        for i in range(1, L):
            for j in range(i + 1, L):
                rec += [jo[s[:i]], jo[s[i:j]], jo[s[j:]], 0]
        return rec

    def pad4(rec):
        return rec + [0] * (-len(rec) % 4)

    def align_prog():
        prog.extend([0] * (-len(prog) % 4))

    TYPE_J, TYPE_T0, TYPE_O, TYPE_R, TYPE_MP = 0, 1, 2, 3, 4
    use_mp = k >= 4
    for stage in range(1, k):
        plist = []
        # gluon currents of length stage+1 (canonical representatives only)
        L = stage + 1
        if L <= k - 1:
            recs = []
            for s in itertools.permutations(range(k), L):
                rep, _ = _canonical(s)
                if rep != s:
                    continue
                rev = tuple(reversed(s))
                recs.append(cur_record(s, jo[s], jo[rev], (-1) ** (L + 1)))
            align_prog()
            plist.append((TYPE_J, L, len(recs), len(prog), len(recs[0])))
            for r in recs:
                prog += r
        # top-line currents with `stage` gluons
        L = stage
        recs = []
        for a in itertools.permutations(range(k), L):
            rec = [oo[a], _mask(a)]
            for i in range(L):
                prev = -1 if i == 0 else oo[a[:i]]
                rec += [prev, jo[a[i:]]]
            recs.append(pad4(rec))
        align_prog()
        plist.append((TYPE_O, L, len(recs), len(prog), len(recs[0])))
        for r in recs:
            prog += r
        # t~ rows of every sequence of length `stage` (not the longest ones
        # when the one-gluon bilinears replace them)
        if not (use_mp and L == k - 1):
            recs = [[ro[b], jo[b]] for b in itertools.permutations(range(k), L)]
            align_prog()
            plist.append((TYPE_R, L, len(recs), len(prog), 2))
            for r in recs:
                prog += r
        # bilinears wtb^T S(e_mu) O(g) of the one-gluon top currents (node:
        # the gluon; item: its 4 (top spin, helicity) entries)
        if use_mp and stage == 2:
            recs = [[oo[(g,)], 0, 0, 0] for g in range(k)]
            align_prog()
            plist.append((TYPE_MP, 1, len(recs), len(prog), 4))
            for r in recs:
                prog += r
        if stage == k - 1:
            recs = []
            for s in perms:
                rep, _ = _canonical(s)
                if rep != s:
                    continue
                rev = tuple(reversed(s))
                recs.append(cur_record(s, pidx[s], pidx[rev], (-1) ** (k + 1)))
            align_prog()
            plist.append((TYPE_T0, k, len(recs), len(prog), len(recs[0])))
            # T0 items write their value straight into the amplitude of the
            # helicity combination: hunpack[sigma][pattern] = gluon helicity bits
            for r in recs:
                prog += r
        parts.append(plist)
    # amplitude records: per ordering, for the splits i = 1..k-1: (O offset,
    # R offset); with the one-gluon bilinears, (O offset, J offset of the
    # suffix) for i = 1
    arec = []
    for s in perms:
        for i in range(1, k):
            arec += [oo[s[:i]], jo[s[i:]] if (use_mp and i == 1) else ro[s[i:]]]
    hpack = []
    hunpack = []
    for s in perms:
        for hg in range(1 << k):
            hpack.append(sum(((hg >> g) & 1) << j for j, g in enumerate(s)))
        for hp in range(1 << k):
            hunpack.append(sum(((hp >> j) & 1) << g for j, g in enumerate(s)))
    # flatten the stage/part descriptors
    pdesc = []
    stage_first = []
    for plist in parts:
        stage_first.append(len(pdesc) // 5)
        for p in plist:
            pdesc += list(p)
    stage_first.append(len(pdesc) // 5)
    hels = helicities(k)
    hidx = {tuple(int(v) for v in h): i for i, h in enumerate(hels)}
    cfg_to_mg = []
    for c in range(1 << (k + 2)):
        hg, ht, htb = c & ((1 << k) - 1), (c >> k) & 1, (c >> (k + 1)) & 1
        h = [0] * (k + 2)
        for q in range(k):
            h[GLUON_PARTICLE[q]] = 1 if (hg >> q) & 1 else -1
        h[2] = 1 if ht else -1
        h[3] = 1 if htb else -1
        cfg_to_mg.append(hidx[tuple(h)])
    return dict(k=k, J_TOTAL=J_TOTAL, O_TOTAL=O_TOTAL, R_TOTAL=R_TOTAL, use_mp=use_mp, prog=prog, pdesc=pdesc,
                stage_first=stage_first, arec=arec, hpack=hpack, hunpack=hunpack,
                jo_ext=[jo[(q,)] for q in range(k)], cfg_to_mg=cfg_to_mg)


def emit_program(k):
    """The program of program_data(k) as a C++ namespace rec<k>."""
    d = program_data(k)
    J_TOTAL, O_TOTAL, R_TOTAL, use_mp = d["J_TOTAL"], d["O_TOTAL"], d["R_TOTAL"], d["use_mp"]
    prog, pdesc, stage_first, arec = d["prog"], d["pdesc"], d["stage_first"], d["arec"]
    hpack, hunpack, cfg_to_mg = d["hpack"], d["hunpack"], d["cfg_to_mg"]
    L = []
    w = L.append
    w(f"namespace rec{k} {{")
    w(f"constexpr int J_TOTAL = {J_TOTAL}, O_TOTAL = {O_TOTAL}, R_TOTAL = {R_TOTAL};")
    w(f"constexpr int NSTAGE = {k - 1}, NPART = {len(pdesc) // 5};")
    w(f"constexpr bool USE_MP = {'true' if use_mp else 'false'};  // one-gluon top-current bilinears")
    body = ", ".join(str(int(v)) for v in prog)
    w(f"__device__ __align__(16) const int prog[{len(prog)}] = {{{body}}};")
    w(f"alignas(16) static const int prog_h[{len(prog)}] = {{{body}}};")
    w(_arr("pdesc", "int", pdesc))
    w(_arr("stage_first", "int", stage_first))
    # the same two tables as compile-time constants (the stage loops)
    w(f"constexpr int pdesc_c[{len(pdesc)}] = {{{', '.join(str(int(v)) for v in pdesc)}}};")
    w(f"constexpr int stage_first_c[{len(stage_first)}] = {{{', '.join(str(int(v)) for v in stage_first)}}};")
    body = ", ".join(str(int(v)) for v in arec)
    w(f"__device__ __align__(8) const int arec[{len(arec)}] = {{{body}}};")
    w(f"alignas(8) static const int arec_h[{len(arec)}] = {{{body}}};")
    w(_arr("hpack", "unsigned char", hpack))
    w(_arr("hunpack", "unsigned char", hunpack))
    w(_arr("jo_ext", "int", d["jo_ext"]))
    w(_arr("cfg_to_mg", "int", cfg_to_mg))
    w("}  // namespace")
    return "\n".join(L)


def write_generated(outdir, ks=(2, 3, 4, 5)):
    import os

    os.makedirs(outdir, exist_ok=True)
    paths = []
    for k in ks:
        path = os.path.join(outdir, f"ttng{k}.cuh")
        src = emit_process_header(k)
        old = open(path).read() if os.path.exists(path) else None
        if old != src:
            with open(path, "w") as f:
                f.write(src)
        paths.append(path)
    return paths
