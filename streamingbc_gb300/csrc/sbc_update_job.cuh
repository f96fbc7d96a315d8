// One root's share of an insertion batch, shared by the single-forest and the
// multi-forest update kernels: a persistent CTA applies every insertion of the
// batch to root r of forest slot A, one job per insertion that joins two
// different levels of r's tree.
#pragma once
#include <climits>
#include "sbc_internal.cuh"

namespace sbc {

template <int NT>
struct UpdSmem {
    LbSmem<NT> lb;
    int64_t dp[NT];
    double wn[NT];
    double wd[NT];
    int fl[NT];
    long long part[3 * (NT / 32) + 3];
    int item, qt, at, st;
    int nscan, nprobe;  // level-2 vertices whose parents are found by scan / by probe
    int mask_ok;        // the current root's level-2 masks hold for this batch
    unsigned long long c1, c2;  // case-1 / case-2 jobs of this CTA (written by thread 0)
};

// A level-2 vertex looks its parents up by binary search (one probe per root
// neighbour) instead of scanning its adjacency when its degree exceeds this
// many times the root's degree; a probe is costed as this many scanned slots.
constexpr int kProbeRatio = 32;

template <int NT, int ILP, bool DECR, bool TOMB>
__device__ __forceinline__ void ascend(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r, int a, int b,
                                       bool moving, int g, bool del, int Lb, int nsteps, int ndown);

// One job: the insertion of edge (a, b) (a the shallower endpoint) on root r,
// or with `del` the deletion of that edge when b keeps another parent (the
// edge is already gone from the adjacency; |d| == 1, levels do not change).
// A deletion is the insertion's sigma-only case with the paths through a
// taken away (diffPath -sigma[a]) and, since b no longer reaches a through
// the adjacency, b's old contribution to a taken out when b is committed
// (removeEdgeWithoutMovementBrandes, src/streamingbc_internal.c:607-868).
template <int NT, int ILP, bool TOMB = false>
__device__ __forceinline__ void run_job(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r,
                                        int a, int b, bool moving, int g, bool del = false)
{
    const int64_t nv = A.G.nv;
    int32_t* D = A.dist + (size_t)r * nv;
    uint8_t* D8 = A.dist8 + (size_t)r * nv;
    uint32_t* D2 = A.dist2 + (size_t)r * d2_words(nv);
    const int64_t* S = A.sigma + (size_t)r * nv;
    const int Lb = D[a] + 1;  // new level of b; equals D[b] when |d| == 1

    if (threadIdx.x == 0) {
        W.st[b] = 1;
        W.dp[b] = del ? -S[a] : S[a];
        W.qd[0] = b;
        W.lvl[0] = 0;
        W.lvl[1] = 1;
        sm.qt = 1;
        sm.at = 0;
        sm.st = 0;
        sm.nscan = 0;
        sm.nprobe = 0;
    }
    __syncthreads();

    // ---------------- descent ----------------
    int step = 0, lo = 0, hi = 1;
    while (lo < hi) {
        const int L = Lb + step;
        const int tag = step + 2;
        // a re-levelling descent compares old distances far from L: one-byte row
        lb_walk<NT, true, ILP, TOMB>(
            A.G, g, DistRow{D, D8, moving ? nullptr : D2, L}, W.qd + lo, hi - lo, nullptr, 0, sm.lb,
            [&](int j, int x, int d) { sm.dp[j] = W.dp[x]; },
            [&](int j, int x, int k, int dk) {
                if (moving ? (dk <= L) : (dk != L + 1)) return;
                int s = W.st[k];
                if (s == 0) {
                    const int old = atomicCAS(&W.st[k], 0, tag);
                    warp_append(&sm.qt, W.qd, k, old == 0);
                    s = old == 0 ? tag : old;
                }
                if ((s & SBC_STEP_MASK) != tag) return;
                atomic_add_i64(&W.dp[k], sm.dp[j]);
            },
            NoPost());
        lo = hi;
        hi = sm.qt;
        ++step;
        if (threadIdx.x == 0) W.lvl[step + 1] = hi;
    }
    const int ndown = hi;
    const int nsteps = step;

    // ---------------- re-level (|d| > 1) ----------------
    if (moving) {
        for (int i = threadIdx.x; i < ndown; i += NT) {
            const int k = W.qd[i];
            const int s = W.st[k];
            const int nl = Lb + (s & SBC_STEP_MASK) - 1;
            if (D[k] != nl) {
                const int old = D[k];
                if (A.lvlhist) {
                    int32_t* H = A.lvlhist + (size_t)r * kHistLevels;
                    if (old != SBC_INF) atomicSub(&H[min(old, kHistLevels - 1)], 1);
                    atomicAdd(&H[min(nl, kHistLevels - 1)], 1);
                }
                if (A.roster) {
                    // k joins level nl's roster (if tracked); its entry in the
                    // roster of its old level goes stale
                    const size_t rb = (size_t)r * kRosterLevels;
                    if (nl >= 2 && nl < kRosterLevels && A.roster_n[rb + nl] <= kRosterCap) {
                        const int p = atomicAdd(&A.roster_n[rb + nl], 1);
                        if (p < kRosterCap) A.roster[(rb + nl) * kRosterCap + p] = k;
                    }
                    if (old >= 2 && old < kRosterLevels && A.roster_n[rb + old] <= kRosterCap)
                        A.roster_dirty[rb + old] = 1;
                }
                D[k] = nl;
                D8[k] = enc_d8(nl);
                set_d2(D2, k, nl);
                W.st[k] = s | SBC_MOVED;
            }
        }
    }
    __syncthreads();
    ascend<NT, ILP, false, TOMB>(A, sm, W, r, a, b, moving, g, del, Lb, nsteps, ndown);
}

// The dependency ascent of a job, from the deepest level its descent touched
// (descent vertices listed by level in W.qd / W.lvl, their st tags, sigma
// changes in W.dp) up to the root, then the reset of the touched scratch.
// DECR: the job is a deletion whose deeper endpoint b lost its last parent
// (movedown below): the moved vertices went DOWN, so an unmoved parent of a
// moved vertex is a parent it gained (its full new weight, not a difference),
// no same-level ex-parent loses a child, and a (not in the descent) loses b's
// old weight, seeded in W.acc[a] and queued when the walk reaches level D[a].
template <int NT, int ILP, bool DECR, bool TOMB>
__device__ __forceinline__ void ascend(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r, int a, int b,
                                       bool moving, int g, bool del, int Lb, int nsteps, int ndown)
{
    const int64_t nv = A.G.nv;
    const uint32_t* M2 = sm.mask_ok ? A.l2mask + (size_t)r * nv : nullptr;
    const int32_t* C1 = sm.mask_ok ? A.l1cand + (size_t)r * kL1Max : nullptr;
    const int n1 = sm.mask_ok ? A.l1n[r] : 0;
    int32_t* D = A.dist + (size_t)r * nv;
    uint8_t* D8 = A.dist8 + (size_t)r * nv;
    uint32_t* D2 = A.dist2 + (size_t)r * d2_words(nv);
    int64_t* S = A.sigma + (size_t)r * nv;
    double* Dl = A.delta + (size_t)r * nv;
    const int root = (int)A.roots[r];
    const int aL = DECR ? D[a] : 0;

    // ---------------- ascent ----------------
    // A parent k's delta gains, per child x, sigma_k * (newdelta_x+1)/newsigma_x,
    // and loses sigma_k * (olddelta_x+1)/oldsigma_x when k is not in the descent
    // (k's sigma is then unchanged) -- except over the inserted edge (a, b),
    // which had no old contribution.  acc[k] therefore sums the unscaled child
    // weights wn = (newdelta+1)/newsigma or wd = wn - (olddelta+1)/oldsigma, and
    // k's sigma multiplies the sum once, when k is committed: the walk over
    // parent edges does no fp64 arithmetic (GB300's fp64 rate is a small
    // fraction of its fp32 rate) and gathers no parent sigma.
    int L = 0;
    // Finalise vertex x of the level being walked: new sigma/delta committed in
    // place, BC += newdelta - olddelta, and its child weights wn, wd returned.
    auto commit = [&](int x, double& wn, double& wd) {
        const int s = W.st[x];
        const bool isDown = (s & SBC_STEP_MASK) != 0;
        const bool mv = (s & SBC_MOVED) != 0;
        const int64_t oS = S[x];
        const double oD = Dl[x];
        const double ac = W.acc[x];
        const int64_t nS = isDown ? (mv ? W.dp[x] : oS + W.dp[x]) : oS;
        const double nD = isDown ? (double)nS * ac : oD + (double)oS * ac;
        wn = (nD + 1.0) / (double)nS;
        wd = oS ? wn - (oD + 1.0) / (double)oS : wn;
        if (x != root) atomicAdd(&A.bc[x], nD - oD);
        S[x] = nS;
        Dl[x] = nD;
        if (!DECR && del && x == b) {
            // a (one level up, not in the descent) loses b's old contribution
            int old = atomicOr(&W.st[a], SBC_ASC);
            if (!(old & SBC_ASC)) W.qa[atomicAdd(&sm.at, 1)] = a;
            atomicAdd(&W.acc[a], wd - wn);
        }
    };
    auto prep = [&](int j, int x, int d) {
        double wn, wd;
        commit(x, wn, wd);
        sm.wn[j] = wn;
        sm.wd[j] = wd;
        sm.fl[j] = ((W.st[x] & SBC_MOVED) ? 1 : 0) | (x == b ? 2 : 0);
    };
    // Child weights of an already committed vertex, kept in its acc/dp slots.
    auto prep_loaded = [&](int j, int x, int d) {
        sm.wn[j] = W.acc[x];
        sm.wd[j] = __longlong_as_double((long long)W.dp[x]);
        sm.fl[j] = ((W.st[x] & SBC_MOVED) ? 1 : 0) | (x == b ? 2 : 0);
    };
    auto parent_edge = [&](int j, int x, int k, int dk) -> bool {
        if (dk != L - 1) return false;
        const int sk = W.st[k];
        const bool kDown = (sk & SBC_STEP_MASK) != 0;
        if (!kDown && !(sk & SBC_ASC)) {
            const int old = atomicOr(&W.st[k], SBC_ASC);
            warp_append(&sm.at, W.qa, k, !(old & SBC_ASC));
        }
        const bool fresh = kDown || (k == a && (sm.fl[j] & 2)) || (DECR && (sm.fl[j] & 1));
        atomicAdd(&W.acc[k], fresh ? sm.wn[j] : sm.wd[j]);
        return true;
    };

    // Pull form for levels 1 and 2.  The parents of a level-1 vertex can only
    // be the root, and those of a level-2 vertex only the root's neighbours, so
    // instead of every walked vertex scanning its (often hub-sized) adjacency
    // for parents, each candidate parent y can scan its own adjacency for
    // walked children c (dist = L and touched) and sum the same child weights
    // (wn[c] if y is in the descent or (y,c) = (a,b), else wd[c]).  The
    // cheaper direction is chosen per level by scanned-slot count; results are
    // the same either way.  Used only where no vertex of the level moved (no
    // same-level ex-parent rule applies).
    // The walked vertices of the level are marked in the worker's bitmap, so a
    // candidate parent tests a neighbour with one (L2-resident) bit instead of
    // gathering its distance and state.
    auto pull_walk = [&](const int32_t* plist, int pn) {
        lb_walk_sum<NT, false, ILP, TOMB>(
            A.G, g, DistRow{D, D8, nullptr, 0}, plist, pn, sm.lb, sm.wn, sm.fl,
            [&](int j, int y, int d) {
                const int sy = W.st[y];
                // a root neighbour whose edge a batched deletion already took
                // is no longer at level 1 (and no parent)
                sm.fl[j] = ((sy & SBC_STEP_MASK) ? 1 : 0) | (y == a ? 2 : 0) | (TOMB && D8[y] != 1 ? 8 : 0);
            },
            [&](int j, int y, int c, int, double& v) -> bool {
                if (!((W.bits[c >> 5] >> (c & 31)) & 1u)) return false;
                const int fl = sm.fl[j];
                if (fl & 8) return false;
                const bool fresh = (fl & 1) || ((fl & 2) && c == b);
                v = fresh ? W.acc[c] : __longlong_as_double((long long)W.dp[c]);
                return true;
            },
            [&](int j, int y) {
                const int fl = sm.fl[j];
                if (!(fl & kSumHit)) return;
                W.acc[y] += sm.wn[j];  // y's only contributions at this level come from this walk
                if (!(fl & 1)) {
                    int old = atomicOr(&W.st[y], SBC_ASC);
                    warp_append(&sm.at, W.qa, y, !(old & SBC_ASC));
                }
            });
    };
    long long pull2_cost = -1;  // scanned slots of a level-2 pull (root's neighbours), computed once

    // Parents of each listed (committed) vertex x at level L, found among
    // candidates cand[0..ncand) -- the root's neighbours (all at level 1) for
    // L = 2, else the roster of level L-1 (entries whose one-byte distance is
    // not L-1 are stale and skipped): each candidate y is looked up in x's
    // sorted adjacency; a hit is a parent, which receives x's child weight
    // (wn[x] if y is in the descent or (y,x) = (a,b), else wd[x]) and is
    // claimed.  Warp per x, lanes over the candidates.
    auto probe_parents = [&](const int32_t* list, int n, const int32_t* cand, int ncand, bool check) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        unsigned cost = 0;
        for (int i = warp; i < n; i += NT / 32) {
            const int x = list[i];
            const int64_t rx = A.G.row[x];
            const int vx = vis_deg(A.G, x, rx, g);
            const double wn = W.acc[x];
            const double wd = __longlong_as_double((long long)W.dp[x]);
            const bool xm = DECR && (W.st[x] & SBC_MOVED);
            for (int t = lane; t < ncand; t += 32) {
                const int y = cand[t];
                if (check && D8[y] != L - 1) continue;
                if (!has_edge<TOMB>(A.G, x, rx, vx, y, g, cost)) continue;
                const int sy = W.st[y];
                const bool yDown = (sy & SBC_STEP_MASK) != 0;
                if (!yDown && !(sy & SBC_ASC)) {
                    const int old = atomicOr(&W.st[y], SBC_ASC);
                    warp_append(&sm.at, W.qa, y, !(old & SBC_ASC));
                }
                atomicAdd(&W.acc[y], (yDown || xm || (y == a && x == b)) ? wn : wd);
            }
        }
        if (cost) atomicAdd(&sm.lb.scanned_e, (unsigned long long)cost);
        __syncthreads();
    };

    // Levels L >= 3 whose level L-1 has a roster: a vertex whose adjacency is
    // much longer than the roster is committed as usual but left out of the
    // walk's scan (its degree is zeroed) and listed at the tail of the level
    // offsets array instead; the probe pass then finds its parents among the
    // roster.  The reference edge counter still counts its full degree.
    const int32_t* rcand = nullptr;
    int rcnt = 0;
    auto prep_div = [&](int j, int x, int& d) {
        prep(j, x, d);
        if (rcand && (long long)d > (long long)kProbeRatio * rcnt) {
            W.acc[x] = sm.wn[j];
            W.dp[x] = (int64_t)__double_as_longlong(sm.wd[j]);
            W.lvl[nv + 1 - warp_reserve(&sm.nprobe, true)] = x;
            atomicAdd(&sm.lb.walked_e, (unsigned long long)d);
            d = 0;
        }
    };
    auto probe_diverted = [&]() {
        const int n = sm.nprobe;
        __syncthreads();
        if (threadIdx.x == 0) sm.nprobe = 0;
        if (n > 0) probe_parents(W.lvl + nv + 2 - n, n, rcand, rcnt, true);
    };

    int ua_lo = 0, ua_hi = 0;
    const int Lmax = Lb + nsteps - 1;
    for (L = Lmax; L >= 0; --L) {
        const int ds = L - Lb;
        const int32_t* dlist = nullptr;
        int dn = 0;
        if (ds >= 0) {
            dlist = W.qd + W.lvl[ds];
            dn = W.lvl[ds + 1] - W.lvl[ds];
        }
        const int next_lo = sm.at;
        const bool pull_ok = L >= 1 && L <= 2 && (!moving || L < Lb);
        rcand = nullptr;
        rcnt = 0;
        if (A.roster && L >= 3 && L - 1 < kRosterLevels) {
            const size_t rb = (size_t)r * kRosterLevels + (L - 1);
            const int c = A.roster_n[rb];
            if (c > 0 && c <= kRosterCap) {
                rcand = A.roster + rb * kRosterCap;
                rcnt = c;
            }
        }
        if (L == 0) {
            // The root alone (if reached): no parents, committing is all.
            if (threadIdx.x == 0 && dn + ua_hi - ua_lo > 0) {
                const int x = dn ? dlist[0] : W.qa[ua_lo];
                double wn, wd;
                commit(x, wn, wd);
                sm.lb.walked_v += 1;
                sm.lb.walked_e += (unsigned)vis_deg(A.G, x, A.G.row[x], g);
            }
            __syncthreads();
        } else {
            // Vertices whose parents the level-1/2 forms below find: the whole
            // level where none of it moved; in a re-levelling job at levels 1-2,
            // the second walk's vertices (ascent-only and same-level ones,
            // none of which moved) once the moved ones have pushed.
            const int32_t* nl1 = dlist;
            const int32_t* nl2 = W.qa + ua_lo;
            int nn1 = dn, nn2 = ua_hi - ua_lo;
            bool near = pull_ok;
            if (!pull_ok && (!moving || DECR)) {
                lb_walk<NT, true, ILP, TOMB>(A.G, g, DistRow{D, D8, D2, L}, dlist, dn, W.qa + ua_lo, ua_hi - ua_lo, sm.lb,
                                       prep_div,
                                       [&](int j, int x, int k, int dk) { parent_edge(j, x, k, dk); }, NoPost());
                probe_diverted();
            } else if (!pull_ok) {
                const int same_lo = sm.st;
                lb_walk<NT, true, ILP, TOMB>(
                    A.G, g, DistRow{D, D8, D2, L}, dlist, dn, nullptr, 0, sm.lb, prep,
                    [&](int j, int x, int k, int dk) {
                        if (parent_edge(j, x, k, dk)) return;
                        if (!(sm.fl[j] & 1) || dk != L) return;
                        // k kept its level and lost the moved vertex x as a child
                        const int sk = W.st[k];
                        if (sk & SBC_STEP_MASK) return;
                        if (!(sk & SBC_ASC)) {
                            const int old = atomicOr(&W.st[k], SBC_ASC);
                            warp_append(&sm.st, W.qs, k, !(old & SBC_ASC));
                        }
                        atomicAdd(&W.acc[k], sm.wd[j] - sm.wn[j]);
                    },
                    NoPost());
                const int same_hi = sm.st;
                const int n2w = ua_hi - ua_lo + same_hi - same_lo;
                // level 2 keeps its scan list after the same-level entries of
                // the queue and its probe list at the queue's end
                if (L == 1 || (L == 2 && (long long)same_hi + 2ll * n2w <= nv)) {
                    near = true;
                    nl1 = W.qa + ua_lo;
                    nn1 = ua_hi - ua_lo;
                    nl2 = W.qs + same_lo;
                    nn2 = same_hi - same_lo;
                } else {
                    lb_walk<NT, true, ILP, TOMB>(A.G, g, DistRow{D, D8, D2, L}, W.qa + ua_lo, ua_hi - ua_lo, W.qs + same_lo,
                                           same_hi - same_lo, sm.lb, prep_div,
                                           [&](int j, int x, int k, int dk) { parent_edge(j, x, k, dk); }, NoPost());
                    probe_diverted();
                }
            }
            if (near) {
                // Commit every vertex x of the level and keep its push weights in
                // its acc/dp slots; count it as traversed (reference counters).
                //   L == 1  the only parent is the root (sigma 1): each x's
                //           contribution is summed straight into the root, no scan.
                //   L == 2  parents are N(x) ∩ N(root).  Per vertex, either scan
                //           N(x) for distance-1 neighbours (push), or, when N(x) is
                //           much longer than N(root), look each root neighbour up
                //           in x's sorted adjacency (probe); or, for the whole
                //           level, let the root's neighbours pull (bitmap test).
                //           The cheapest plan by scanned slots is taken.
                const int64_t rrow = A.G.row[root];
                const int rdeg = vis_deg(A.G, root, rrow, g);
                const bool rootDown = (W.st[root] & SBC_STEP_MASK) != 0;
                long long push_cost = 0, mixed_cost = 0;
                double root_sum = 0.0;
                const int qbase = sm.st;  // free tail of the same-level queue holds the two lists
                for (int i = threadIdx.x; i < nn1 + nn2; i += NT) {
                    const int x = i < nn1 ? nl1[i] : nl2[i - nn1];
                    // loads that need only x, issued before commit's stores
                    const int64_t rx = A.G.row[x];
                    const int xd0 = A.G.deg0[x], xd = A.G.deg[x];
                    const unsigned m0 = (L == 2 && M2) ? M2[x] : 0u;
                    double wn, wd;
                    commit(x, wn, wd);
                    W.acc[x] = wn;
                    W.dp[x] = (int64_t)__double_as_longlong(wd);
                    const int dx = (xd0 == xd || g == INT_MAX) ? xd : vis_deg(A.G, x, rx, g);
                    push_cost += dx;
                    if (L == 1) {
                        root_sum += (rootDown || (root == a && x == b)) ? wn : wd;
                    } else if (L == 2 && M2) {
                        // parents from the mask (edges older than the batch),
                        // plus this batch's edges visible here that reach a root
                        // neighbour (level 1)
                        unsigned m = m0;
                        for (int sl = xd0; sl < dx; ++sl) {
                            const int z = A.G.col[rx + sl];
                            if (D8[z] == 1)
                                for (int q = 0; q < n1; ++q)
                                    if (C1[q] == z) m |= 1u << q;
                        }
                        while (m) {
                            const int q = __ffs(m) - 1;
                            m &= m - 1;
                            const int y = C1[q];
                            const int sy = W.st[y];
                            const bool yDown = (sy & SBC_STEP_MASK) != 0;
                            // a root neighbour is claimed by the first of its
                            // many children; the others see the flag already
                            if (!yDown && !(sy & SBC_ASC)) {
                                const int old = atomicOr(&W.st[y], SBC_ASC);
                                warp_append(&sm.at, W.qa, y, !(old & SBC_ASC));
                            }
                            atomicAdd(&W.acc[y], (yDown || (y == a && x == b)) ? wn : wd);
                        }
                    } else if (L == 2) {
                        atomicOr(&W.bits[x >> 5], 1u << (x & 31));
                        const bool probe = (long long)dx > (long long)kProbeRatio * rdeg;
                        const int pp = warp_reserve(&sm.nprobe, probe);
                        const int ps = warp_reserve(&sm.nscan, !probe);
                        if (probe) {
                            W.qs[nv - 1 - pp] = x;
                            mixed_cost += (long long)kProbeRatio * rdeg;
                        } else {
                            W.qs[qbase + ps] = x;
                            mixed_cost += dx;
                        }
                    }
                }
                block_sum3<NT>(push_cost, mixed_cost, root_sum, sm.part);
                if (threadIdx.x == 0) {
                    sm.lb.walked_v += (unsigned)(nn1 + nn2);
                    sm.lb.walked_e += (unsigned long long)push_cost;
                }
                if (L == 1) {
                    if (threadIdx.x == 0 && nn1 + nn2 > 0) {
                        W.acc[root] += root_sum;
                        if (!rootDown) {
                            int old = atomicOr(&W.st[root], SBC_ASC);
                            if (!(old & SBC_ASC)) W.qa[atomicAdd(&sm.at, 1)] = root;
                        }
                    }
                    __syncthreads();
                } else if (L == 2 && nn1 + nn2 > 0 && M2) {
                    __syncthreads();  // every parent took its share in the commit loop
                } else if (L == 2 && nn1 + nn2 > 0) {
                    if (pull2_cost < 0) {
                        long long c = 0;
                        for (int i = threadIdx.x; i < rdeg; i += NT) {
                            const int y = A.G.col[rrow + i];
                            c += vis_deg(A.G, y, A.G.row[y], g);
                        }
                        pull2_cost = block_sum<NT>(c, sm.part);
                    }
                    if (pull2_cost < mixed_cost) {
                        pull_walk(A.G.col + rrow, rdeg);
                    } else {
                        const int nscan = sm.nscan, nprobe = sm.nprobe;
                        lb_walk<NT, false, ILP, TOMB>(A.G, g, DistRow{D, D8, D2, L}, W.qs + qbase, nscan, nullptr, 0, sm.lb,
                                                prep_loaded,
                                           [&](int j, int x, int k, int dk) { parent_edge(j, x, k, dk); }, NoPost());
                        probe_parents(W.qs + nv - nprobe, nprobe, A.G.col + rrow, rdeg, TOMB);
                    }
                    for (int i = threadIdx.x; i < nn1 + nn2; i += NT) {
                        const int x = i < nn1 ? nl1[i] : nl2[i - nn1];
                        W.bits[x >> 5] = 0u;  // words hold only this level's marks
                    }
                    __syncthreads();
                }
            }
        }
        if (DECR && L == aL + 1) {
            // a lost b's old weight (seeded in acc[a]): walked at its level
            if (threadIdx.x == 0) {
                const int old = atomicOr(&W.st[a], SBC_ASC);
                if (!(old & SBC_ASC)) W.qa[atomicAdd(&sm.at, 1)] = a;
            }
            __syncthreads();
        }
        ua_lo = next_lo;
        ua_hi = sm.at;
        if (L <= Lb && ua_lo == ua_hi && (!DECR || L <= aL + 1)) break;
    }

    // ---------------- reset touched scratch ----------------
    const int na = sm.at, ns = sm.st;
    for (int i = threadIdx.x; i < ndown; i += NT) {
        const int k = W.qd[i];
        W.st[k] = 0;
        W.dp[k] = 0;
        W.acc[k] = 0.0;
    }
    for (int i = threadIdx.x; i < na; i += NT) {
        const int k = W.qa[i];
        W.st[k] = 0;
        W.dp[k] = 0;  // may hold a push weight (pull-form levels)
        W.acc[k] = 0.0;
    }
    for (int i = threadIdx.x; i < ns; i += NT) {
        const int k = W.qs[i];
        W.st[k] = 0;
        W.dp[k] = 0;  // may hold a child weight (probed levels)
        W.acc[k] = 0.0;
    }
    __syncthreads();
}

// Applies the batch's insertions in order to root r of slot A: each live
// insertion (append code > 0) whose endpoints sit on different levels is one
// job, |d| == 1 (case 1) or |d| > 1 / one endpoint unreachable (case 2).
template <int NT, int ILP>
__device__ __forceinline__ void process_root(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r,
                                             bool all_visible)
{
    const int32_t* D = A.dist + (size_t)r * A.G.nv;
    // level-2 masks hold for the whole batch unless one of its insertions
    // changes the root's own neighbour list
    bool mk = A.l2mask && A.l1n[r] >= 0;
    if (mk) {
        const int root = (int)A.roots[r];
        int hit = 0;
        for (int i = threadIdx.x; i < A.nins; i += NT)
            if (A.ins_ok[i] > 0 && (A.ins_u[i] == root || A.ins_v[i] == root)) hit = 1;
        mk = !__syncthreads_or(hit);
    }
    if (threadIdx.x == 0) sm.mask_ok = mk ? 1 : 0;
    __syncthreads();
    for (int i = 0; i < A.nins; ++i) {
        if (A.ins_ok[i] <= 0) continue;
        const int u = A.ins_u[i], v = A.ins_v[i];
        const int du = D[u], dv = D[v];
        if (du == dv) continue;  // same level, or both unreachable
        const int b = du > dv ? u : v;
        const int a = du > dv ? v : u;
        const int db = du > dv ? du : dv, da = du > dv ? dv : du;
        const bool moving = (db == SBC_INF) || (db - da > 1);
        if (threadIdx.x == 0) {
            if (moving) sm.c2 += 1;
            else sm.c1 += 1;
        }
        const unsigned long long walked0 = sm.lb.walked_v;  // read before run_job's first barrier
        run_job<NT, ILP>(A, sm, W, r, a, b, moving, all_visible ? INT_MAX : i);
        if (A.cost_log && threadIdx.x == 0)
            A.cost_log[(size_t)r * A.nins + i] = (int32_t)min(sm.lb.walked_v - walked0, (unsigned long long)INT_MAX);
    }
}

// Deletion worklist entries: root index | kLostRoot when the deeper endpoint
// has no parent left.
constexpr int kLostRoot = 0x40000000;

// Scratch states of a move-down job (bits outside SBC_STEP_MASK, SBC_MOVED and
// SBC_ASC; cleared before its ascent).
constexpr int kDecUp = 0x04000000;    // candidate with a parent outside the affected set
constexpr int kDecAff = 0x20000000;   // in the affected set: its level grows
constexpr int kDecCand = 0x40000000;  // child of an affected vertex, tested for another parent

// Affected sets larger than this are left to a recompute of the root.
__device__ __forceinline__ int movedown_cap(int64_t nv) { return (int)max((int64_t)1024, nv / 16); }

// Block-wide minimum (op 0) or maximum (op 1) of v over the threads; *cell is
// a shared int the block may overwrite.
template <int NT>
__device__ __forceinline__ int block_minmax(int v, int* cell, int op)
{
    __syncthreads();
    if (threadIdx.x == 0) *cell = op ? INT_MIN : INT_MAX;
    __syncthreads();
    if (op ? v > INT_MIN : v < INT_MAX) {
        if (op) atomicMax(cell, v);
        else atomicMin(cell, v);
    }
    __syncthreads();
    const int out = *cell;
    __syncthreads();
    return out;
}

// Deletion of (a, b) (already gone from the adjacency) on root r where b, one
// level below a, had a as its only parent: b and possibly part of its subtree
// move down (moveDownTreeBrandes, src/streamingbc_internal.c:880-1401, whose
// result disagrees with a recompute; this one is exact):
//   1. affected set X, by old level from b: a child of X all of whose parents
//      are in X joins X; the other children ("boundary") keep their level and
//      lose the paths through their parents in X (sigma change -sum sigma).
//   2. new levels of X: 1 + the lowest unaffected neighbour, then relaxed
//      inside X in level order (unit-weight Dijkstra); none: unreachable.
//   3. level by level from D[b] + 1: sigma of the X vertices from their new
//      parents, and the sigma changes of the boundary pushed down to the
//      unaffected children (an X vertex never parents an unaffected one, since
//      its new level exceeds its old one and neighbours' old levels differ by
//      at most one), listing every changed vertex by level as a descent does.
//   4. X re-levelled (unreachable ones leave BC and get sigma 0), then the
//      shared ascent with the move-down rules.
// Returns false, with the root's state untouched and the scratch clean, when
// X outgrows movedown_cap: the root is then recomputed.
template <int NT, int ILP, bool TOMB>
__device__ bool movedown(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r, int a, int b, int g)
{
    const int64_t nv = A.G.nv;
    int32_t* D = A.dist + (size_t)r * nv;
    uint8_t* D8 = A.dist8 + (size_t)r * nv;
    uint32_t* D2 = A.dist2 + (size_t)r * d2_words(nv);
    int64_t* S = A.sigma + (size_t)r * nv;
    double* Dl = A.delta + (size_t)r * nv;
    const int root = (int)A.roots[r];
    const int lb = D[b];
    const double wb = (Dl[b] + 1.0) / (double)S[b];  // b's old weight, which a loses
    const DistRow row{D, D8, nullptr, 0};
    auto noprep = [](int, int, int) {};
    if (threadIdx.x == 0) {
        W.st[b] = kDecAff;
        W.qs[0] = b;
        sm.st = 1;  // X, in W.qs
        sm.at = 0;  // candidates, in W.qa
        sm.qt = 0;
    }
    __syncthreads();

    // ---- 1. affected set ----
    int lo = 0, hi = 1, l = lb;
    bool over = false;
    while (lo < hi) {
        const int c_lo = sm.at;
        lb_walk<NT, false, ILP, TOMB>(A.G, g, row, W.qs + lo, hi - lo, nullptr, 0, sm.lb, noprep,
                                [&](int, int, int k, int dk) {
                                    if (dk != l + 1 || W.st[k] != 0) return;
                                    const int old = atomicCAS(&W.st[k], 0, kDecCand);
                                    warp_append(&sm.at, W.qa, k, old == 0);
                                },
                                NoPost());
        const int c_hi = sm.at;
        lb_walk<NT, false, ILP, TOMB>(A.G, g, row, W.qa + c_lo, c_hi - c_lo, nullptr, 0, sm.lb, noprep,
                                [&](int, int k, int y, int dy) {
                                    if (dy != l) return;
                                    if (W.st[y] & kDecAff) atomic_add_i64(&W.dp[k], S[y]);
                                    else if (!(W.st[k] & kDecUp)) atomicOr(&W.st[k], kDecUp);
                                },
                                NoPost());
        for (int i = c_lo + threadIdx.x; i < c_hi; i += NT) {
            const int k = W.qa[i];
            const bool in = !(W.st[k] & kDecUp);
            if (in) {
                W.st[k] = kDecAff;
                W.dp[k] = 0;
            } else {
                W.dp[k] = -W.dp[k];  // boundary: sigma change so far
            }
            warp_append(&sm.st, W.qs, k, in);
        }
        __syncthreads();
        lo = hi;
        hi = sm.st;
        ++l;
        if (hi > movedown_cap(nv)) {
            over = true;
            break;
        }
    }
    const int nx = sm.st, nc = sm.at;
    if (over) {
        for (int i = threadIdx.x; i < nx; i += NT) {
            W.st[W.qs[i]] = 0;
            W.dp[W.qs[i]] = 0;
        }
        for (int i = threadIdx.x; i < nc; i += NT) {
            W.st[W.qa[i]] = 0;
            W.dp[W.qa[i]] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) sm.st = sm.at = 0;
        __syncthreads();
        return false;
    }

    // ---- 2. new levels of X (held in the step bits; SBC_STEP_MASK = none) ----
    for (int i = threadIdx.x; i < nx; i += NT) W.st[W.qs[i]] = kDecAff | SBC_STEP_MASK;
    __syncthreads();
    lb_walk<NT, false, ILP, TOMB>(A.G, g, row, W.qs, nx, nullptr, 0, sm.lb, noprep,
                            [&](int, int x, int y, int dy) {
                                if (dy == SBC_INF || (W.st[y] & kDecAff)) return;
                                const int want = kDecAff | (dy + 1);
                                if (want < W.st[x]) atomicMin(&W.st[x], want);
                            },
                            NoPost());
    int tl = INT_MAX;
    for (int i = threadIdx.x; i < nx; i += NT) tl = min(tl, W.st[W.qs[i]] & SBC_STEP_MASK);
    int L = block_minmax<NT>(tl, &sm.nprobe, 0);
    int tmax = 0;
    while (L < SBC_STEP_MASK) {
        tmax = L;
        if (threadIdx.x == 0) sm.qt = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < nx; i += NT) {
            const int x = W.qs[i];
            warp_append(&sm.qt, W.qd, x, (W.st[x] & SBC_STEP_MASK) == L);
        }
        __syncthreads();
        lb_walk<NT, false, ILP, TOMB>(A.G, g, row, W.qd, sm.qt, nullptr, 0, sm.lb, noprep,
                                [&](int, int, int z, int) {
                                    const int sz = W.st[z];
                                    if ((sz & kDecAff) && (sz & SBC_STEP_MASK) > L + 1)
                                        atomicMin(&W.st[z], kDecAff | (L + 1));
                                },
                                NoPost());
        tl = INT_MAX;
        for (int i = threadIdx.x; i < nx; i += NT) {
            const int t = W.st[W.qs[i]] & SBC_STEP_MASK;
            if (t > L) tl = min(tl, t);
        }
        L = block_minmax<NT>(tl, &sm.nprobe, 0);
    }

    // ---- 3. sigma by level ----
    const int Lb = lb + 1;  // no vertex above this level changes
    for (int i = threadIdx.x; i < nx; i += NT) {
        const int x = W.qs[i];
        const int t = W.st[x] & SBC_STEP_MASK;
        W.st[x] = kDecAff | (t == SBC_STEP_MASK ? 0 : t - Lb + 1);  // tag of the new level; 0: unreachable
    }
    int um = INT_MIN;
    for (int i = threadIdx.x; i < nc; i += NT) {
        const int k = W.qa[i];
        if (!(W.st[k] & kDecAff)) um = max(um, D[k]);
    }
    const int Lend = max(block_minmax<NT>(um, &sm.nprobe, 1), tmax);
    if (threadIdx.x == 0) {
        sm.qt = 0;
        W.lvl[0] = 0;
    }
    __syncthreads();
    int step = 0;
    for (int Lc = Lb;; ++Lc, ++step) {
        const int tag = step + 1;
        const int p_hi = sm.qt;  // vertices pushed to this level by the previous one
        __syncthreads();
        for (int i = threadIdx.x; i < nx; i += NT) {
            const int x = W.qs[i];
            warp_append(&sm.qt, W.qd, x, (W.st[x] & SBC_STEP_MASK) == tag);
        }
        __syncthreads();
        const int x_hi = sm.qt;
        __syncthreads();
        for (int i = threadIdx.x; i < nc; i += NT) {
            const int k = W.qa[i];
            const int s = W.st[k];
            const bool take = !(s & kDecAff) && !(s & SBC_STEP_MASK) && D[k] == Lc;
            if (take) W.st[k] = s | tag;
            warp_append(&sm.qt, W.qd, k, take);
        }
        __syncthreads();
        const int end = sm.qt;
        const int seg_lo = W.lvl[step];
        if (threadIdx.x == 0) W.lvl[step + 1] = end;
        // X vertices of this level: sigma from the new parents one level up
        lb_walk<NT, false, ILP, TOMB>(A.G, g, row, W.qd + p_hi, x_hi - p_hi, nullptr, 0, sm.lb, noprep,
                                [&](int, int x, int y, int dy) {
                                    const int sy = W.st[y];
                                    int ly;
                                    int64_t sg;
                                    if (sy & kDecAff) {
                                        const int ty = sy & SBC_STEP_MASK;
                                        if (ty == 0) return;
                                        ly = Lb + ty - 1;
                                        sg = W.dp[y];
                                    } else {
                                        ly = dy;
                                        sg = S[y] + ((sy & SBC_STEP_MASK) ? W.dp[y] : 0);
                                    }
                                    if (ly == Lc - 1) atomic_add_i64(&W.dp[x], sg);
                                },
                                NoPost());
        // unaffected vertices of this level: their sigma changes to their
        // unaffected children (never to an X vertex)
        lb_walk<NT, false, ILP, TOMB>(
            A.G, g, row, W.qd + seg_lo, p_hi - seg_lo, W.qd + x_hi, end - x_hi, sm.lb,
            [&](int j, int x, int) { sm.dp[j] = W.dp[x]; },
            [&](int j, int, int k, int dk) {
                if (dk != Lc + 1) return;
                int s = W.st[k];
                if (s & kDecAff) return;
                if (!(s & SBC_STEP_MASK)) {
                    const int old = atomicCAS(&W.st[k], s, s | (tag + 1));
                    warp_append(&sm.qt, W.qd, k, old == s);
                    s = old == s ? (s | (tag + 1)) : old;
                }
                if ((s & SBC_STEP_MASK) != tag + 1) return;
                atomic_add_i64(&W.dp[k], sm.dp[j]);
            },
            NoPost());
        if (sm.qt == end && Lc >= Lend) {
            ++step;
            break;
        }
    }
    const int nsteps = step, ndown = sm.qt;

    // ---- 4. re-level X, then the ascent ----
    for (int i = threadIdx.x; i < nc; i += NT) {
        const int k = W.qa[i];
        const int s = W.st[k];
        if (!(s & kDecAff)) W.st[k] = s & SBC_STEP_MASK;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nx; i += NT) {
        const int x = W.qs[i];
        const int tag = W.st[x] & SBC_STEP_MASK;
        const int old = D[x];
        const int nl = tag ? Lb + tag - 1 : SBC_INF;
        if (A.lvlhist) {
            int32_t* H = A.lvlhist + (size_t)r * kHistLevels;
            atomicSub(&H[min(old, kHistLevels - 1)], 1);
            if (tag) atomicAdd(&H[min(nl, kHistLevels - 1)], 1);
        }
        if (A.roster) {
            const size_t rb = (size_t)r * kRosterLevels;
            if (tag && nl >= 2 && nl < kRosterLevels && A.roster_n[rb + nl] <= kRosterCap) {
                const int p = atomicAdd(&A.roster_n[rb + nl], 1);
                if (p < kRosterCap) A.roster[(rb + nl) * kRosterCap + p] = x;
            }
            if (old >= 2 && old < kRosterLevels && A.roster_n[rb + old] <= kRosterCap) A.roster_dirty[rb + old] = 1;
        }
        D[x] = nl;
        D8[x] = enc_d8(nl);
        set_d2(D2, x, nl);
        if (tag) {
            W.st[x] = tag | SBC_MOVED;
        } else {
            // unreachable now: out of BC, no paths
            if (x != root) atomicAdd(&A.bc[x], -Dl[x]);
            S[x] = 0;
            Dl[x] = 0.0;
            W.st[x] = 0;
            W.dp[x] = 0;
        }
    }
    if (threadIdx.x == 0) {
        W.acc[a] = -wb;
        sm.at = 0;
        sm.st = nx;  // X stays listed in W.qs for the final reset
        sm.nscan = sm.nprobe = 0;
    }
    __syncthreads();
    ascend<NT, ILP, true, TOMB>(A, sm, W, r, a, b, true, g, true, Lb, nsteps, ndown);
    return true;
}

// The deletion of (u, v) on root r.  lost: the deeper endpoint has no parent
// left (the classify step's split); such a root moves down, or, when that
// fails, joins the recompute list mov.
template <int NT, int ILP>
__device__ __forceinline__ void process_deletion(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r,
                                                 int u, int v, bool lost, int* mov, int* nmov)
{
    const int32_t* D = A.dist + (size_t)r * A.G.nv;
    const int du = D[u], dv = D[v];
    if (du == dv) return;
    // the masks were brought up to date with the removal before this launch
    if (threadIdx.x == 0) {
        if (!lost) sm.c1 += 1;
        sm.mask_ok = (A.l2mask && A.l1n[r] >= 0) ? 1 : 0;
    }
    __syncthreads();
    const int a = du < dv ? u : v, b = du < dv ? v : u;
    if (!lost) {
        run_job<NT, ILP>(A, sm, W, r, a, b, false, INT_MAX, true);
    } else if (!movedown<NT, ILP, false>(A, sm, W, r, a, b, INT_MAX)) {
        if (threadIdx.x == 0) mov[atomicAdd(nmov, 1)] = r;
    }
}

// Every deletion of a batch applied in order to root r.  The batch's removed
// slots are still in place, marked (slot_live<true>), so deletion i's jobs see
// the graph without the edges of deletions 0..i, as one-at-a-time deletions
// would.  Per deletion, on the root's current levels: endpoints on one level
// change nothing; else the deeper endpoint b keeps a parent (sigma-only job)
// or not (move-down).  Without move-down (or when it outgrows its cap) the
// root's dependencies (exact for the graph before deletion i) leave BC, the
// root joins the dirty list and skips the batch's later deletions; it is
// recomputed on the final graph after the launch.  The level-2 masks describe
// the graph before the batch and are not used.
template <int NT, int ILP>
__device__ __forceinline__ void process_root_deletions(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r,
                                                       bool move_down, int* dirty, int* dlist, int* dcnt)
{
    const int64_t nv = A.G.nv;
    const int32_t* D = A.dist + (size_t)r * nv;
    if (threadIdx.x == 0) sm.mask_ok = 0;
    __syncthreads();
    for (int i = 0; i < A.nins; ++i) {
        if (A.ins_ok[i] != 1) continue;
        const int u = A.ins_u[i], v = A.ins_v[i];
        const int du = D[u], dv = D[v];
        if (du == dv) continue;
        const int a = du < dv ? u : v, b = du < dv ? v : u;
        const int lb = max(du, dv);
        const int64_t rb = A.G.row[b];
        const int db = A.G.deg[b];
        int has = 0;
        for (int s = threadIdx.x; s < db && !has; s += NT)
            if (D[A.G.col[rb + s]] == lb - 1 && slot_live<true>(A.G, rb + s, i)) has = 1;
        if (__syncthreads_or(has)) {
            if (threadIdx.x == 0) sm.c1 += 1;
            run_job<NT, ILP, true>(A, sm, W, r, a, b, false, i, true);
            continue;
        }
        if (threadIdx.x == 0) sm.c2 += 1;
        if (move_down && movedown<NT, ILP, true>(A, sm, W, r, a, b, i)) continue;
        const int root = (int)A.roots[r];
        const double* Dl = A.delta + (size_t)r * nv;
        for (int64_t x = threadIdx.x; x < nv; x += NT) {
            const double d = Dl[x];
            if (d != 0.0 && x != root) atomicAdd(&A.bc[x], -d);
        }
        if (threadIdx.x == 0) {
            dirty[r] = 1;
            dlist[atomicAdd(dcnt, 1)] = r;
        }
        __syncthreads();
        break;
    }
}

// Zeroes the CTA's traversal and case counters (thread 0, before the first barrier).
template <int NT>
__device__ __forceinline__ void reset_counters(UpdSmem<NT>& sm)
{
    if (threadIdx.x == 0) sm.lb.walked_v = sm.lb.walked_e = sm.lb.scanned_e = sm.c1 = sm.c2 = 0;
}

// Adds the CTA's traversal and case counters into counters[0..4].
template <int NT>
__device__ __forceinline__ void flush_counters(UpdSmem<NT>& sm, unsigned long long* counters)
{
    if (threadIdx.x == 0) {
        atomicAdd(&counters[0], sm.lb.walked_v);
        atomicAdd(&counters[1], sm.lb.walked_e);
        atomicAdd(&counters[2], sm.c1);
        atomicAdd(&counters[3], sm.c2);
        atomicAdd(&counters[4], sm.lb.scanned_e);
    }
}

}  // namespace sbc
