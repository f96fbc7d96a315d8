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

// One job: the insertion of edge (a, b) (a the shallower endpoint) on root r,
// or with `del` the deletion of that edge when b keeps another parent (the
// edge is already gone from the adjacency; |d| == 1, levels do not change).
// A deletion is the insertion's sigma-only case with the paths through a
// taken away (diffPath -sigma[a]) and, since b no longer reaches a through
// the adjacency, b's old contribution to a taken out when b is committed
// (removeEdgeWithoutMovementBrandes, src/streamingbc_internal.c:607-868).
template <int NT, int ILP>
__device__ __forceinline__ void run_job(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r,
                                        int a, int b, bool moving, int g, bool del = false)
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
        lb_walk<NT, true, ILP>(
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
        if (del && x == b) {
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
        const bool fresh = kDown || (k == a && (sm.fl[j] & 2));
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
        lb_walk_sum<NT, false, ILP>(
            A.G, g, DistRow{D, D8, nullptr, 0}, plist, pn, sm.lb, sm.wn, sm.fl,
            [&](int j, int y, int d) {
                const int sy = W.st[y];
                sm.fl[j] = ((sy & SBC_STEP_MASK) ? 1 : 0) | (y == a ? 2 : 0);
            },
            [&](int j, int y, int c, int, double& v) -> bool {
                if (!((W.bits[c >> 5] >> (c & 31)) & 1u)) return false;
                const int fl = sm.fl[j];
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
            for (int t = lane; t < ncand; t += 32) {
                const int y = cand[t];
                if (check && D8[y] != L - 1) continue;
                if (!has_edge(A.G, x, rx, vx, y, cost)) continue;
                const int sy = W.st[y];
                const bool yDown = (sy & SBC_STEP_MASK) != 0;
                if (!yDown && !(sy & SBC_ASC)) {
                    const int old = atomicOr(&W.st[y], SBC_ASC);
                    warp_append(&sm.at, W.qa, y, !(old & SBC_ASC));
                }
                atomicAdd(&W.acc[y], (yDown || (y == a && x == b)) ? wn : wd);
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
            if (!pull_ok && !moving) {
                lb_walk<NT, true, ILP>(A.G, g, DistRow{D, D8, D2, L}, dlist, dn, W.qa + ua_lo, ua_hi - ua_lo, sm.lb,
                                       prep_div,
                                       [&](int j, int x, int k, int dk) { parent_edge(j, x, k, dk); }, NoPost());
                probe_diverted();
            } else if (!pull_ok) {
                const int same_lo = sm.st;
                lb_walk<NT, true, ILP>(
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
                    lb_walk<NT, true, ILP>(A.G, g, DistRow{D, D8, D2, L}, W.qa + ua_lo, ua_hi - ua_lo, W.qs + same_lo,
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
                            const bool yDown = (W.st[y] & SBC_STEP_MASK) != 0;
                            if (!yDown) {
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
                        lb_walk<NT, false, ILP>(A.G, g, DistRow{D, D8, D2, L}, W.qs + qbase, nscan, nullptr, 0, sm.lb,
                                                prep_loaded,
                                           [&](int j, int x, int k, int dk) { parent_edge(j, x, k, dk); }, NoPost());
                        probe_parents(W.qs + nv - nprobe, nprobe, A.G.col + rrow, rdeg, false);
                    }
                    for (int i = threadIdx.x; i < nn1 + nn2; i += NT) {
                        const int x = i < nn1 ? nl1[i] : nl2[i - nn1];
                        W.bits[x >> 5] = 0u;  // words hold only this level's marks
                    }
                    __syncthreads();
                }
            }
        }
        ua_lo = next_lo;
        ua_hi = sm.at;
        if (L <= Lb && ua_lo == ua_hi) break;
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

// The deletion of (u, v) on root r, which keeps a parent of the deeper
// endpoint (the classify step sends the other roots to a recompute).
template <int NT, int ILP>
__device__ __forceinline__ void process_deletion(const ForestSlot& A, UpdSmem<NT>& sm, const Scratch& W, int r,
                                                 int u, int v)
{
    const int32_t* D = A.dist + (size_t)r * A.G.nv;
    const int du = D[u], dv = D[v];
    if (du == dv) return;
    // the masks were brought up to date with the removal before this launch
    if (threadIdx.x == 0) {
        sm.c1 += 1;
        sm.mask_ok = (A.l2mask && A.l1n[r] >= 0) ? 1 : 0;
    }
    __syncthreads();
    run_job<NT, ILP>(A, sm, W, r, du < dv ? u : v, du < dv ? v : u, false, INT_MAX, true);
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
