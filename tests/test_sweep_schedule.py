"""The wavefront sweep's schedule (turbulentbl_gb300/csrc/tbl_sweep.cu,
k_sweep), checked on the CPU.

A model of the kernel's index arithmetic -- positions per lane and step,
the 32-row block lag, the first and last steps T0/T1 of each warp, the
two-steps-ahead operand ring, the plane-to-plane ring and the wait targets
-- runs every warp in global step order.  Data from other warps is read
from the state as of the end of the previous step, so a read of something
not yet produced, or already overwritten, gives a different result from the
sequential lexicographic sweep the reference performs
(dnstbl2/dnstbl.f90:830-868 Gauss-Seidel, :1022-1042 and :1115-1135 block
SSOR), which the model also runs.  The model asserts that every wait
targets a step its producer completes, that every index stays inside its
buffer and that every operand slot holds the chunk a lane reads from it.
The same model with a block lag one step short, or with the one-position
row lag on a 4-row grid (where the kernel keeps a lag of a chunk), must
disagree with the sequential sweep.

The point arithmetic is a*b + c in both runs (the schedule, not the
rounding, is under test).
"""
import random

import pytest

CH = 4     # points per lane and step in FP64 (8 in FP32: run(..., ch=8))
KG = 4     # planes (warps) per CTA
RING = 4   # plane-to-plane slots
XR = 8     # slots of the cluster ring (the kernel's XR_SLOTS)
OPB = 16   # operand buffer elements per lane, 4 CH (position q at q % OPB)


def fma(a, b, c):
    return a * b + c


def run(mode, nx, J, K_list, plag, jb_rows=0, nib=1, seed=0, blag_delta=0, ch=4, xk=False, xr=XR):
    """One sweep of mode 0 (Gauss-Seidel), 1 (forward SSOR) or 2 (backward
    SSOR) over slabs of K_list planes, J span rows and nx points per line,
    by the kernel's schedule with row lag plag (and block lag changed by
    blag_delta) and sequentially.  Returns (points that differ, last step,
    counts of the waits checked).  ch: points per lane and step.  xk: the
    CTAs of a slab column form a cluster and hand the plane below over
    through a ring of XR slots in the upper CTA's shared memory (st.async
    into the slot, mbarrier phases), instead of global memory and flags;
    xr: its slots."""
    CH, OPB = ch, 4 * ch
    rnd = random.Random(seed)
    sx = ((nx + 7) + 7) // 8 * 8
    C = (nx - 2) // CH + 1
    assert CH * C <= sx
    CB = (C + nib - 1) // nib
    nblk = (C + CB - 1) // CB if mode != 0 else 1
    if mode == 0:
        nib_ = 1
    else:
        nib_ = nib
    P = len(K_list)
    ny = J + 2
    njb = (J + 31) // 32
    # CTA table
    ctas = []
    slabs = []
    bn = 1
    # slab columns (same slab and row block, kg = 0..nkc-1) are consecutive
    # CTAs -- a cluster in the kernel -- with idle CTAs above a short slab
    nkc = max((K + KG - 1) // KG for K in K_list)
    for r, K in enumerate(K_list):
        slabs.append((bn, K))
        bn += K
        nkg = (K + KG - 1) // KG
        base = len(ctas)
        for jb in range(njb):
            for kg in range(nkc):
                live = kg < nkg
                ctas.append(dict(slab=r, jb=jb, kg=kg,
                                 up_j=base + (jb - 1) * nkc + kg if live and jb > 0 else -1,
                                 up_k=base + jb * nkc + (kg - 1) if live and kg > 0 else -1,
                                 dn_j=live and jb < njb - 1, dn_k=live and kg < nkg - 1))
    xk = xk and 2 <= nkc <= 8

    def publishes(cidx, wid):
        """The kernel's rule for the device-scope progress flag of a warp."""
        c = ctas[cidx]
        j_reader = c['dn_j'] and not (mode != 0 and jb_rows > 0 and (32 * (c['jb'] + 1)) % jb_rows == 0)
        return j_reader or (wid == KG - 1 and c['dn_k'] and not xk)
    nz = bn + 1
    ps = sx * ny
    vol = ps * nz
    cj, ck, ci, p2 = 0.3, 0.2, 0.4, 0.15
    if mode == 2:
        p0 = 1.7
    inp = [rnd.uniform(-1, 1) for _ in range(vol)]     # PRE (GS) / RH (FWD, BWD)
    F = [rnd.uniform(-1, 1) for _ in range(vol)]       # GS field (old values); bnd at i = 0
    halo_in = {}  # (slab) -> plane values for kidx == 0 GS reads (the slab below's top plane snapshot)
    for r in range(P):
        halo_in[r] = [rnd.uniform(-1, 1) for _ in range(ps)]

    def idx(i, j, k):
        assert 0 <= i < sx, i
        assert 0 <= j < ny
        assert 0 <= k < nz
        return i + sx * (j + ny * k)

    # ---------------- sequential reference (lexicographic per slab)
    Fseq = list(F)
    RHseq = list(inp)
    OUTseq = [0.0] * vol
    for r, (bnr, K) in enumerate(slabs):
        for bi in range(nblk if mode != 0 else 1):
            c_lo = bi * CB if mode != 0 else 0
            c_hi = min(C, c_lo + CB) - 1 if mode != 0 else C - 1
            Q = CH * (c_hi - c_lo + 1)
            ibase = CH * c_hi + CH - 1 if mode == 2 else CH * c_lo
            idir = -1 if mode == 2 else 1
            for kl in range(K):
                kidx = K - 1 - kl if mode == 2 else kl
                k = bnr + kidx
                for jl in range(J):
                    jblk0 = (jl // jb_rows) * jb_rows if (mode != 0 and jb_rows > 0) else 0
                    jr = jl - jblk0
                    jidx = J - 1 - jl if mode == 2 else jl
                    j = 1 + jidx
                    carry = 0.0
                    bnd = F[idx(0, j, k)] if mode == 0 else 0.0
                    for q in range(Q):
                        i = ibase + idir * q
                        cur = inp[idx(i, j, k)]
                        if mode == 2:
                            cur = p0 * cur
                        inr = 1 <= i <= nx - 2
                        # wrap (GS, last row reads row 1 new)
                        if mode == 0 and j == ny - 2:
                            cur = fma(p2, Fseq[idx(i, 1, k)], cur)
                        # k input
                        if mode == 0:
                            if kidx == 0 and r > 0:
                                pk = halo_in[r][i + sx * j]
                            else:
                                pk = Fseq[idx(i, j, k - 1)]
                        else:
                            kin_zero = (kidx == 0) if mode == 1 else (kidx == K - 1)
                            if kin_zero:
                                pk = 0.0
                            else:
                                pk = (RHseq if mode == 1 else OUTseq)[idx(i, j, k - 1 if mode == 1 else k + 1)]
                        # j input
                        if mode == 0:
                            jm = ny - 2 if j == 1 else j - 1
                            pj = Fseq[idx(i, jm, k)]
                        else:
                            if jr == 0:
                                pj = 0.0
                            else:
                                pj = (RHseq if mode == 1 else OUTseq)[idx(i, j - 1 if mode == 1 else j + 1, k)]
                        cur = fma(ck, pk, cur)
                        nv = fma(cj, pj, cur)
                        if q == 0:
                            carry = 0.0
                        if inr:
                            carry = fma(ci, carry, nv)
                            o = carry
                        else:
                            o = bnd if (mode == 0 and i == 0) else 0.0
                            carry = o
                        if mode == 0:
                            if inr:
                                Fseq[idx(i, j, k)] = o
                        elif mode == 1:
                            RHseq[idx(i, j, k)] = o
                        else:
                            OUTseq[idx(i, j, k)] = o
    # ---------------- the kernel's schedule
    G = list(F)           # GS field written by the sweep
    RH = list(inp)        # FWD in place
    OUT = [0.0] * vol
    wstep = {}            # global location -> step written
    warps = []
    for ci_, cta in enumerate(ctas):
        for by in range(nib_):
            for wid in range(KG):
                warps.append((ci_, by, wid))
    st = {}
    ring = {}   # (cta, by, wid, slot) -> (step, [lane][e])
    xring = {}  # cluster hand-off: (consumer cta, by, slot) -> (index pushed, [lane][e])
    maxT = 0
    info = {}
    for (cidx, by, wid) in warps:
        cta = ctas[cidx]
        bnr, K = slabs[cta['slab']]
        c_lo = by * CB if mode != 0 else 0
        c_hi = min(C, c_lo + CB) - 1 if mode != 0 else C - 1
        Cl = c_hi - c_lo + 1
        if Cl <= 0:
            continue
        kl = KG * cta['kg'] + wid
        if kl >= K:
            continue
        jblk0 = (32 * cta['jb'] // jb_rows) * jb_rows if (mode != 0 and jb_rows > 0) else 0
        bj = (32 * cta['jb'] - jblk0) >> 5
        blag = (31 * plag + 2 * CH - 1) // CH + blag_delta
        lane_last = min(32 * cta['jb'] + 31, J - 1) - 32 * cta['jb']
        Q = CH * Cl
        T0 = kl + blag * bj
        T1 = T0 + (Q - 1 + plag * lane_last) // CH
        info[(cidx, by, wid)] = dict(T0=T0, T1=T1, kl=kl, K=K, bnr=bnr, c_lo=c_lo, c_hi=c_hi, Cl=Cl, Q=Q,
                                     jblk0=jblk0, lane_last=lane_last)
        maxT = max(maxT, T1)
        st[(cidx, by, wid)] = dict(last=[[0.0] * CH for _ in range(32)], carry=[0.0] * 32,
                                   slots={}, done=-1)
    # issue_raw bookkeeping: slots[(lane, element)] = (chunk, step, position held)
    def chunk_of(inf, lane, ts):
        return (CH * (ts - inf['T0']) - plag * lane + CH - 1) // CH

    def issue(w, ts):
        inf = info[w]
        cta = ctas[w[0]]
        for lane in range(32):
            jl = 32 * cta['jb'] + lane
            if not (jl < J):
                continue
            ac = chunk_of(inf, lane, ts)
            if ts <= inf['T1'] and 0 <= ac < inf['Cl']:
                i0 = CH * (inf['c_hi'] - ac if mode == 2 else inf['c_lo'] + ac)
                assert i0 % CH == 0 and i0 + CH <= sx
                base = (CH * ac) & (OPB - 1)
                assert base % CH == 0  # 16-byte aligned destination
                for t in range(CH):
                    pos = CH * ac + (CH - 1 - t if mode == 2 else t)
                    st[w]['slots'][(lane, base + t)] = (ac, ts, pos)

    for w in info:
        issue(w, info[w]['T0'])
        issue(w, info[w]['T0'] + 1)

    checks = dict(j_wait=0, k_wait=0, fast=0, x_push=0)
    for T in range(0, maxT + 1):
        snapG, snapRH, snapOUT = list(G), list(RH), list(OUT)
        snap_ring = dict(ring)
        snap_xring = dict(xring)
        snap_done = {w: st[w]['done'] for w in st}
        for w in info:
            inf = info[w]
            if not (inf['T0'] <= T <= inf['T1']):
                continue
            cidx, by, wid = w
            cta = ctas[cidx]
            bnr, K = inf['bnr'], inf['K']
            kl = inf['kl']
            T0, T1 = inf['T0'], inf['T1']
            tend_k = T1 - 1
            # waits: producers must have completed the target steps (in the snapshot)
            if cta['up_j'] >= 0 and 32 * cta['jb'] != inf['jblk0'] and T - T0 < inf['Cl']:
                up = (cta['up_j'], by, wid)
                assert publishes(cta['up_j'], wid), "j producer does not publish its progress"
                tgt = T - 1
                assert tgt <= info[up]['T1'], ("j target beyond producer's last step", tgt, info[up]['T1'])
                assert snap_done[up] >= tgt, ("j producer behind", T, snap_done[up], tgt)
                checks['j_wait'] += 1
            if kl > 0:
                tgt = min(T - 1, tend_k)
                if wid > 0:
                    up = (cidx, by, wid - 1)
                else:
                    up = (cta['up_k'], by, KG - 1)
                    assert cta['up_k'] // nkc == cidx // nkc, "k producer outside the slab column"
                    assert xk or publishes(cta['up_k'], KG - 1), "k producer does not publish its progress"
                assert info[up]['T1'] == tend_k, ("tend_k", info[up]['T1'], tend_k)
                assert snap_done[up] >= tgt
                checks['k_wait'] += 1
            outs = [[0.0] * CH for _ in range(32)]
            lanes = []
            for lane in range(32):
                jl = 32 * cta['jb'] + lane
                jr = jl - inf['jblk0']
                line_ok = jl < J
                jidx = J - 1 - jl if mode == 2 else jl
                kidx = K - 1 - kl if mode == 2 else kl
                j = 1 + max(0, min(jidx, J - 1))
                k = bnr + kidx
                jm = ny - 2 if j == 1 else j - 1
                jp = 1 if j == ny - 2 else j + 1
                dl = plag * lane
                qb = CH * (T - T0) - dl
                aT = chunk_of(inf, lane, T)
                ibase = CH * inf['c_hi'] + CH - 1 if mode == 2 else CH * inf['c_lo']
                idir = -1 if mode == 2 else 1
                act = [line_ok and 0 <= qb + e < inf['Q'] for e in range(CH)]
                ix = [ibase + idir * (qb + e) for e in range(CH)]
                inr = [1 <= x <= nx - 2 for x in ix]
                cur = [0.0] * CH
                for e in range(CH):
                    if act[e]:
                        q = qb + e
                        assert 0 <= ix[e] < sx
                        assert (q // CH) in (aT, aT - 1)
                        el = (q ^ (CH - 1) if mode == 2 else q) & (OPB - 1)
                        ent = st[w]['slots'].get((lane, el))
                        assert ent is not None and ent[0] == (q // CH) and ent[2] == q, ("buffer content", ent, q, T)
                        assert ent[1] <= T
                        r_ = inp[idx(ix[e], j, k)]  # operands are inputs, never overwritten before use
                        if mode == 1:
                            r_ = snapRH[idx(ix[e], j, k)]
                            assert r_ == inp[idx(ix[e], j, k)], "FWD operand overwritten before its read"
                        cur[e] = p0 * r_ if mode == 2 else r_
                lanes.append(dict(lane=lane, jr=jr, line_ok=line_ok, j=j, k=k, jm=jm, jp=jp, kidx=kidx, qb=qb,
                                  act=act, ix=ix, inr=inr, cur=cur, jidx=jidx))
            # the kernel's specialised step: every lane has a line and all its
            # points are interior positions of the block, not the first one
            ibase_w = CH * inf['c_hi'] + CH - 1 if mode == 2 else CH * inf['c_lo']
            qlo = max(1, ibase_w - (nx - 2) if mode == 2 else 1 - ibase_w)
            qhi = min(inf['Q'] - 1, ibase_w - 1 if mode == 2 else nx - 2 - ibase_w)
            q0 = CH * (T - T0)
            full_warp = plag == 1 and 32 * cta['jb'] + 31 < J
            if full_warp and q0 - 31 >= qlo and q0 + CH - 1 <= qhi:
                checks['fast'] += 1
                for L in lanes:
                    assert L['line_ok'] and all(L['act']) and all(L['inr'])
                    assert all(L['qb'] + e != 0 for e in range(CH))
            # pk, pj0, wrap
            for L in lanes:
                lane = L['lane']
                act, ix, j, k = L['act'], L['ix'], L['j'], L['k']
                pk = [0.0] * CH
                if wid > 0:
                    key = (cidx, by, wid - 1, (T - 1) % RING)
                    ent = snap_ring.get(key)
                    for e in range(CH):
                        if act[e]:
                            assert ent is not None and ent[0] == T - 1, ("ring", ent and ent[0], T - 1)
                            pk[e] = ent[1][lane][e]
                elif xk and cta['up_k'] >= 0:
                    # ring slot (T - T0) % XR holds the producer's (T - T0)-th push, its step T - 1
                    xu = T - T0
                    ent = snap_xring.get((cidx, by, xu % xr))
                    assert ent is not None and ent[0] == xu, ("cluster ring", ent and ent[0], xu)
                    for e in range(CH):
                        if act[e]:
                            pk[e] = ent[1][lane][e]
                else:
                    for e in range(CH):
                        if not act[e]:
                            continue
                        if mode == 0:
                            if L['kidx'] == 0 and ctas[cidx]['slab'] > 0:
                                pk[e] = halo_in[ctas[cidx]['slab']][ix[e] + sx * j]
                            else:
                                pk[e] = snapG[idx(ix[e], j, k - 1)]
                        else:
                            kin_zero = (L['kidx'] == 0) if mode == 1 else (L['kidx'] == K - 1)
                            if not kin_zero:
                                kk = k - 1 if mode == 1 else k + 1
                                pk[e] = (snapRH if mode == 1 else snapOUT)[idx(ix[e], j, kk)]
                L['pk'] = pk
                pj0 = [0.0] * CH
                if lane == 0:
                    if mode != 0:
                        assert L['qb'] % CH == 0 or not any(act)
                    for e in range(CH):
                        if not act[e]:
                            continue
                        if mode == 0:
                            pj0[e] = snapG[idx(ix[e], L['jm'], k)]
                            # row 1 reading the last row: that row must not have been written yet
                            if L['jidx'] == 0:
                                assert wstep.get(('G', idx(ix[e], L['jm'], k)), 10 ** 9) > T, "wrap row read after its write"
                        else:
                            if L['jr'] != 0:
                                jj = j - 1 if mode == 1 else j + 1
                                pj0[e] = (snapRH if mode == 1 else snapOUT)[idx(ix[e], jj, k)]
                L['pj0'] = pj0
                if mode == 0 and L['jp'] == 1:
                    for e in range(CH):
                        if act[e]:
                            loc = idx(ix[e], 1, k)
                            assert wstep.get(('G', loc), -1) < T or not L['inr'][e], "wrap reads row 1 not yet written"
                            L['cur'][e] = fma(p2, snapG[loc], L['cur'][e])
                for e in range(CH):
                    L['cur'][e] = fma(ck, pk[e], L['cur'][e])
            # the point loop with shuffles (lockstep over lanes)
            last = st[w]['last']
            out = [[0.0] * CH for _ in range(32)]
            for e in range(CH):
                srcs = []
                for L in lanes:
                    lane = L['lane']
                    if plag == 1:
                        srcs.append(last[lane][CH - 1] if e == 0 else out[lane][e - 1])
                    else:
                        srcs.append(last[lane][e])
                for L in lanes:
                    lane = L['lane']
                    pj = srcs[lane - 1] if lane > 0 else srcs[0]
                    if lane == 0:
                        pj = L['pj0'][e]
                    nv = fma(cj, pj, L['cur'][e])
                    out[lane][e] = 0.0
                    if L['act'][e]:
                        if L['qb'] + e == 0:
                            st[w]['carry'][lane] = 0.0
                        if L['inr'][e]:
                            st[w]['carry'][lane] = fma(ci, st[w]['carry'][lane], nv)
                            out[lane][e] = st[w]['carry'][lane]
                        else:
                            bnd = F[idx(0, L['j'], L['k'])] if mode == 0 else 0.0
                            out[lane][e] = bnd if (mode == 0 and L['ix'][e] == 0) else 0.0
                            st[w]['carry'][lane] = out[lane][e]
            st[w]['last'] = [list(o) for o in out]
            # ring
            has_down = wid < KG - 1 and kl + 1 < K
            if has_down:
                ring[(cidx, by, wid, T % RING)] = (T, [list(o) for o in out])
            if xk and wid == KG - 1 and cta['dn_k']:
                # push to the CTA above: the consumer released this slot's
                # previous use (index xu - XR, read at its step T0c + xu - XR)
                cons = (cidx + 1, by, 0)
                assert ctas[cidx + 1]['up_k'] == cidx and (cidx + 1) // nkc == cidx // nkc
                xu = T - T0
                assert info[cons]['T0'] == T0 + 1 and info[cons]['T1'] == T1 + 1
                if xu >= xr:
                    assert snap_done[cons] >= info[cons]['T0'] + xu - xr, "slot overwritten before its release"
                    # the release is sent only for slots written again
                    assert (xu - xr) + xr <= info[cons]['T1'] - info[cons]['T0']
                xring[(cidx + 1, by, xu % xr)] = (xu, [list(o) for o in out])
                checks['x_push'] += 1
            # stores
            for L in lanes:
                for e in range(CH):
                    if L['act'][e] and (mode != 0 or L['inr'][e]):
                        loc = idx(L['ix'][e], L['j'], L['k'])
                        if mode == 0:
                            G[loc] = out[L['lane']][e]
                            wstep[('G', loc)] = T
                        elif mode == 1:
                            RH[loc] = out[L['lane']][e]
                        else:
                            OUT[loc] = out[L['lane']][e]
            st[w]['done'] = T
            issue(w, T + 2)
    # compare
    ref = Fseq if mode == 0 else (RHseq if mode == 1 else OUTseq)
    got = G if mode == 0 else (RH if mode == 1 else OUT)
    bad = sum(1 for a, b in zip(ref, got) if a != b)
    return bad, maxT, checks


def kernel_plag(J, ch=CH):
    """The row lag the host picks for a grid with J span rows (base_args):
    one position, or a whole chunk when J <= ch (the Gauss-Seidel wrap row
    would otherwise read row 1's value in the step that writes it)."""
    return ch if J <= ch else 1


def _cases():
    out = []
    for mode in (0, 1, 2):
        for nx in (8, 12, 17, 23):
            for J in (4, 5, 6, 9, 33, 40, 70):
                for Ks in ((3,), (5, 4), (9,), (2, 6, 5)):
                    opts = ((0, 1),) if mode == 0 else ((0, 1), (32, 1), (0, 2), (32, 3))
                    for jb_rows, nib in opts:
                        out.append((mode, nx, J, Ks, jb_rows, nib))
    rnd = random.Random(7)
    return rnd.sample(out, 160)


@pytest.mark.parametrize("mode,nx,J,Ks,jb_rows,nib", _cases())
def test_schedule_reproduces_the_sequential_sweep(mode, nx, J, Ks, jb_rows, nib):
    bad, _, checks = run(mode, nx, J, list(Ks), kernel_plag(J), jb_rows, nib)
    assert bad == 0
    if J > 32 and not (mode != 0 and jb_rows):
        assert checks["j_wait"] > 0  # blocks below the first wait on the block above


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_chunk_lag_schedule_also_holds(mode):
    """plag = CH is the schedule of grids with 4 span rows or fewer; it is
    valid on every grid."""
    for J in (5, 33, 40):
        assert run(mode, 12, J, [5, 4], CH)[0] == 0


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_a_block_lag_one_step_short_breaks_the_order(mode):
    bad, _, _ = run(mode, 12, 40, [3], 1, blag_delta=-1)
    assert bad > 0


def test_one_position_lag_breaks_the_gs_wrap_on_four_rows():
    assert run(0, 12, 4, [3], 1)[0] > 0
    assert run(0, 12, 4, [3], CH)[0] == 0
    assert run(1, 12, 4, [3], 1)[0] == 0  # SSOR has no wrap row


def test_model_mirrors_the_kernel_source():
    """The formulas this model restates, as they appear in the kernel and its
    host glue (a change to either side must be made to both)."""
    from pathlib import Path
    src = (Path(__file__).resolve().parents[1] / "turbulentbl_gb300" / "csrc" / "tbl_sweep.cu").read_text()
    for line in (
        "const int blag = (31 * plag + 2 * CH - 1) / CH;",
        "const int T0 = kl + blag * bj;",
        "const int T1 = T0 + (Q - 1 + plag * lane_last) / CH;",
        "const int dl = plag * lane;",
        "auto chunk_of = [&](int ts) { return (CH * (ts - T0) - dl + CH - 1) >> LG; };",
        "template <typename Val> constexpr int sweep_ch() { return sizeof(Val) == 4 ? 8 : 4; }",
        "constexpr int OPB = 4 * CH;",
        "const int qb = CH * (T - T0) - dl;",
        "const Val r = opb[(MODE == SW_BWD ? (q ^ (CH - 1)) : q) & (OPB - 1)];",
        "Val* dst = opb + ((CH * ac) & (OPB - 1));",
        "const int qlo = max(1, MODE == SW_BWD ? ibase - (g.nx - 2) : 1 - ibase);",
        "const int qhi = min(Q - 1, MODE == SW_BWD ? ibase - 1 : g.nx - 2 - ibase);",
        "const bool full_warp = plag == 1 && 32 * cta.jb + 31 < J;",
        "const bool j_reader = cta.dn_j && !(MODE != SW_GS && a.jb_rows > 0 && (32 * (cta.jb + 1)) % a.jb_rows == 0);",
        "const bool publish = j_reader || (wid == KG - 1 && cta.dn_k && !xk);",
        "c.up_j = live && jb > 0 ? base + (jb - 1) * nkc + kg : -1;",
        "c.up_k = live && kg > 0 ? base + jb * nkc + (kg - 1) : -1;",
        "c.dn_j = live && jb < njb - 1 ? 1 : 0;",
        "c.dn_k = live && kg < nkg - 1 ? 1 : 0;",
        "constexpr int XR_SLOTS = 8;",
        "const bool xprod = xk && wid == KG - 1 && cta.dn_k;",
        "const bool xcons = xk && wid == 0 && cta.up_k >= 0;",
        "const int xu = T - T0;",
        "if (xcons && !mbar_wait(&s_full[xu % XR], (unsigned)(xu / XR) & 1u)) abort = 1;",
        "if (lane == 0 && xu + XR <= T1 - T0) {",
        "if (xu >= XR && !mbar_wait(&s_empty[xu % XR], (unsigned)(xu / XR - 1) & 1u)) abort = 1;",
        "if (nkc >= 2 && nkc <= 8) {",
        "const bool ok = (full_warp && q0 - 31 >= qlo && q0 + CH - 1 <= qhi) ? step(T, std::true_type{})",
        "a.plag = h->g.ny - 2 <= sweep_ch<T>() ? sweep_ch<T>() : 1;",
        "constexpr int RING = 4;",

    ):
        assert line in src, line


@pytest.mark.parametrize("mode,nib", [(0, 1), (1, 1), (2, 1), (1, 2), (2, 2)])
def test_specialised_steps_reproduce_the_sequential_sweep(mode, nib):
    """Lines long enough that the 32-lane warps run steps with every point
    interior (the kernel's specialised step), on two full row blocks."""
    bad, _, checks = run(mode, 83, 64, [5, 4], kernel_plag(64), 0, nib)
    assert bad == 0
    assert checks["fast"] > 0


def _cluster_cases():
    out = []
    for mode in (0, 1, 2):
        for nx, J, Ks, nib, ch in [(23, 40, (5, 4), 1, 4), (17, 9, (9,), 1, 4), (12, 33, (2, 6, 5), 1, 4),
                                   (40, 70, (13, 4), 1, 4), (83, 64, (16, 15), 1, 4), (40, 33, (9, 3), 2, 4),
                                   (83, 64, (5, 4), 1, 8), (30, 9, (13, 4), 1, 8), (150, 40, (9,), 2, 8)]:
            if mode == 0 and nib > 1:
                continue
            out.append((mode, nx, J, Ks, nib, ch))
    return out


@pytest.mark.parametrize("mode,nx,J,Ks,nib,ch", _cluster_cases())
def test_cluster_hand_off_reproduces_the_sequential_sweep(mode, nx, J, Ks, nib, ch):
    """Plane groups of a slab column as one cluster: the plane below reaches
    warp 0 of the upper CTAs through the XR-slot ring (slot and phase of
    every push and read, release before reuse), also with idle CTAs above a
    short slab; same steps, same values."""
    plag = kernel_plag(J, ch)
    bad, last, checks = run(mode, nx, J, list(Ks), plag, 0, nib, ch=ch, xk=True)
    assert bad == 0
    assert checks["x_push"] > 0
    assert last == run(mode, nx, J, list(Ks), plag, 0, nib, ch=ch)[1]


def test_a_one_slot_cluster_ring_would_be_overwritten_before_its_read():
    """The consumer runs one step behind its producer, so a single slot is
    refilled before it is read (the kernel's ring has 8)."""
    with pytest.raises(AssertionError, match="slot overwritten"):
        run(1, 23, 40, [5, 4], 1, xk=True, xr=1)
    assert run(1, 23, 40, [5, 4], 1, xk=True, xr=2)[0] == 0


def _cases8():
    out = []
    for mode in (0, 1, 2):
        for nx, J, Ks, nib in [(83, 64, (5, 4), 1), (40, 33, (3, 6), 1), (83, 64, (5, 4), 2), (17, 5, (3,), 1),
                               (23, 40, (2, 6, 5), 1), (30, 9, (4,), 1), (21, 8, (3, 2), 1), (150, 40, (5,), 1)]:
            if mode == 0 and nib > 1:
                continue
            out.append((mode, nx, J, Ks, nib))
    return out


@pytest.mark.parametrize("mode,nx,J,Ks,nib", _cases8())
def test_eight_point_steps_reproduce_the_sequential_sweep(mode, nx, J, Ks, nib):
    """The FP32 sweeps' 8 points per lane and step, with the row lag the host
    picks for them (a whole chunk up to 8 span rows)."""
    bad, _, checks = run(mode, nx, J, list(Ks), kernel_plag(J, 8), 0, nib, ch=8)
    assert bad == 0
    if nx > 70 and J >= 32 and nib == 1:
        assert checks["fast"] > 0


def test_one_position_lag_needs_more_rows_than_points_per_step():
    """With 8 points per step the Gauss-Seidel wrap breaks up to 8 span rows
    under a one-position lag, and holds from 9."""
    assert run(0, 23, 8, [3, 4], 1, ch=8)[0] > 0
    assert run(0, 23, 8, [3, 4], 8, ch=8)[0] == 0
    assert run(0, 23, 9, [3, 4], 1, ch=8)[0] == 0
