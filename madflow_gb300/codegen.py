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


def _jname(seq):
    return "J_" + "".join(str(g) for g in seq)


def emit_amplitudes(k):
    """CUDA source of ``ttng<k>_amps<T>``: all colour-ordered partial
    amplitudes of one event for one helicity."""
    L = []
    w = L.append
    w(f"// Generated by madflow_gb300.codegen for {process_name(k)}: {math.factorial(k)} colour orderings.")
    w("template <class T>")
    w(f"MF_D void ttng{k}_amps(const EvData<T, {k}>& ev, const W4<T>* g, const W4<T>& wt,")
    w("                                             const W4<T>& wtb, cx<T>* A) {")
    # J table: lengths 2..k-1, canonical representatives
    made = set()
    for length in range(2, k):
        for seq in itertools.permutations(range(k), length):
            rep, sgn = _canonical(seq)
            if rep in made:
                continue
            made.add(rep)
            s = _mask(rep)
            w(f"  W4<T> {_jname(rep)};")
            w("  {")
            w("    W4<T> a3 = w4zero<T>(), a4 = w4zero<T>();")
            for i in range(1, length):
                left, right = rep[:i], rep[i:]
                w(f"    vvv_add<T>({_jref(left)}, ev.Qg[{_mask(left)}], {_jref(right)}, ev.Qg[{_mask(right)}], a3);")
            for i in range(1, length):
                for j in range(i + 1, length):
                    w(f"    vvvv_add<T>({_jref(rep[:i])}, {_jref(rep[i:j])}, {_jref(rep[j:])}, a4);")
            w(f"    {_jname(rep)} = combine<T>(ev.gv3[{s}], a3, ev.gv4[{s}], a4);")
            w("  }")
    w("  #pragma unroll")
    w(f"  for (int i = 0; i < {math.factorial(k)}; ++i) A[i] = cx<T>{{T(0), T(0)}};")
    # full-length gluon currents contracted with the bare quark line: A(sigma) += amp * wtb^T S(J(sigma)) wt
    perms = permutations(k)
    pidx = {p: i for i, p in enumerate(perms)}
    done = set()
    full = _mask(range(k))
    for sig in perms:
        rep, sgn = _canonical(sig)
        if rep in done:
            continue
        done.add(rep)
        w("  {")
        w("    W4<T> a3 = w4zero<T>(), a4 = w4zero<T>();")
        for i in range(1, k):
            left, right = rep[:i], rep[i:]
            w(f"    vvv_add<T>({_jref(left)}, ev.Qg[{_mask(left)}], {_jref(right)}, ev.Qg[{_mask(right)}], a3);")
        for i in range(1, k):
            for j in range(i + 1, k):
                w(f"    vvvv_add<T>({_jref(rep[:i])}, {_jref(rep[i:j])}, {_jref(rep[j:])}, a4);")
        w(f"    W4<T> Jf = combine<T>(ev.gv3[{full}], a3, ev.gv4[{full}], a4);")
        w("    cx<T> t = sandwich<T>(wtb, Jf, wt);")
        rev = tuple(reversed(rep))
        w(f"    A[{pidx[rep]}] += t;")
        if rev != rep:
            rsgn = (-1) ** (k + 1)
            w(f"    A[{pidx[rev]}] {'+=' if rsgn > 0 else '-='} t;")
        w("  }")
    # DFS over prefixes of the top-quark line
    def dfs(prefix, depth_names):
        # prefix: tuple of gluons attached so far (len >= 1); emit O(prefix)
        m = len(prefix)
        oname = "O_" + "".join(str(g) for g in prefix)
        w("  " * m + "{")
        ind = "  " * (m + 1)
        w(f"{ind}W4<T> y = w4zero<T>();")
        names = depth_names + [oname]
        for i in range(m):
            a_name = names[i]  # O(prefix[:i]) (i = 0 -> wt)
            b = prefix[i:]
            w(f"{ind}sv_add<T>({_jref(b)}, {a_name}, y);")
        w(f"{ind}W4<T> {oname} = topprop<T>(ev.Qt[{_mask(prefix)}], ev.mt, ev.tden[{_mask(prefix)}], y);")
        if m == k - 1:
            last = [g for g in range(k) if g not in prefix][0]
            sig = prefix + (last,)
            w(f"{ind}{{")
            w(f"{ind}  cx<T> acc = cx<T>{{T(0), T(0)}};")
            for i in range(1, k):
                o_name = names[i] if i < len(names) else oname
                if i == m:
                    o_name = oname
                else:
                    o_name = names[i]
                b = sig[i:]
                w(f"{ind}  acc += sandwich<T>(wtb, {_jref(b)}, {o_name});")
            w(f"{ind}  A[{pidx[sig]}] += acc;")
            w(f"{ind}}}")
        else:
            for g in range(k):
                if g not in prefix:
                    dfs(prefix + (g,), names)
        w("  " * m + "}")

    for g in range(k):
        dfs((g,), ["wt"])
    w("}")
    return "\n".join(L)


def _jref(seq):
    """Expression for J(seq): external for length 1, table entry (with the
    reflection sign) otherwise."""
    if len(seq) == 1:
        return f"g[{seq[0]}]"
    rep, sgn = _canonical(tuple(seq))
    return _jname(rep) if sgn > 0 else f"neg<T>({_jname(rep)})"


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
    L.append(f"__constant__ float colour_num[{n * n}] = {{")
    for r in num:
        L.append("  " + ", ".join(f"{float(v)!r}f" for v in r) + ",")
    L.append("};")
    L.append(f"__constant__ signed char hel[{len(hels)}][{k + 2}] = {{")
    for h in hels:
        L.append("  {" + ", ".join(str(int(v)) for v in h) + "},")
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
    L.append(emit_amplitudes(k))
    return "\n".join(L) + "\n"


def write_generated(outdir, ks=(2, 3, 4)):
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
