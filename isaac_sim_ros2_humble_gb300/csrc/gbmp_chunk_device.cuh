// gbmp_chunk_device.cuh -- validation of consecutive states of an edge by chunks
// (device routines shared by the edge-validation kernel, gbmp_chunk.cu, and the
// planner's edge checks, gbmp_rrtc_device.cuh).
//
// The interpolated states of one edge lie millimetres apart, so the obstacles near one
// state are the obstacles near its neighbours.  A warp takes K consecutive states of
// one edge (a chunk) and
//   A. runs the FK of all K states together (the joint-local transforms spread over the
//      lanes, then one lane per pose row of each state walking the chain), keeping the
//      link poses in shared memory, and bounds the centre of every sphere group (a
//      link's bounding sphere) over the chunk by an axis-aligned box;
//   B. turns each box into a swept group sphere: centre = box centre, radius = half the
//      box diagonal + the group radius (which already carries kBroadMargin);
//   C. runs the broad phase ONCE for the chunk: the bounding sphere of every run of 32
//      obstacles (scenes store obstacles in spatially compact runs) against the swept
//      group spheres, then the obstacles of the runs some group touches against those
//      groups, keeping the obstacles that touch any (with the group mask) in a per-warp
//      candidate list;
//   D. walks the states in order and tests each state's robot spheres exactly against
//      the candidates only (the same narrow tests as warp_collide_culled), then its
//      self-collision pairs, stopping at the first colliding state.
// Because the swept spheres enclose every per-state group sphere, the candidate list
// holds every obstacle any state of the chunk can touch, and the narrow tests are the
// exact ones: verdicts and first-hit indices equal the per-state kernel's.  A chunk
// whose candidates overflow the list falls back to the per-state routine.
#pragma once

#include "gbmp_internal.h"

namespace gbmp {

constexpr int kChunkCands = 64;
constexpr int kChunkPairs = 64;

struct ChunkScratch {
    float *lpK;       // link poses of the chunk's states [K][L*12]
    float *locK;      // joint-local transforms of the chunk's states [K][L*12]
    float4 *sgb;      // swept group spheres (x, y, z, R) [G]
    float *sgA;       // |c|^2 - R^2 of each swept sphere
    unsigned *cl;     // candidate obstacle indices
    unsigned *cm;     // their group masks
    int *pl;          // enabled group pairs whose swept spheres overlap (lpair indices)
    int *nl;          // the spheres of the groups in `need`, in sphere order
};

// Per-warp shared memory of the chunk kernel: the link poses of the chunk, then one
// region used twice: by the joint-local transforms while the FK runs (phase A), and
// afterwards by the swept spheres, candidate lists and the parts of WarpScratch the
// per-state tests use (sphere centres, group spheres, candidates).  Group arrays are
// sized by the robot's group count.  For the 8-DOF benchmark arm this is 6.9 KB per warp
// (11 KB without the sharing), which leaves room for larger scenes.
__host__ __device__ inline size_t smem_chunk_rest(const DevRobot &R) {
    return align16(sizeof(float4) * R.G) + align16(sizeof(float) * R.G) + 2 * align16(sizeof(unsigned) * kChunkCands) +
           align16(sizeof(int) * kChunkPairs) + align16(sizeof(int) * R.S) + align16(sizeof(float4) * R.S) +
           align16(sizeof(float4) * R.G) + align16(sizeof(float) * R.G) + 2 * align16(sizeof(int) * kWarp);
}

__host__ __device__ inline size_t smem_chunk_bytes(const DevRobot &R, int K) {
    const size_t poses = align16(sizeof(float) * 12 * R.L * K), rest = smem_chunk_rest(R);
    return poses + (poses > rest ? poses : rest);
}

__device__ inline void carve_chunk(unsigned char *base, const DevRobot &R, int K, int warp, ChunkScratch &c,
                                   WarpScratch &w) {
    unsigned char *p = base + smem_chunk_bytes(R, K) * warp;
    size_t off = 0;
    c.lpK = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * 12 * R.L * K);
    c.locK = reinterpret_cast<float *>(p + off);   // shares the region carved below
    c.sgb = reinterpret_cast<float4 *>(p + off); off += align16(sizeof(float4) * R.G);
    c.sgA = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * R.G);
    c.cl = reinterpret_cast<unsigned *>(p + off); off += align16(sizeof(unsigned) * kChunkCands);
    c.cm = reinterpret_cast<unsigned *>(p + off); off += align16(sizeof(unsigned) * kChunkCands);
    c.pl = reinterpret_cast<int *>(p + off); off += align16(sizeof(int) * kChunkPairs);
    c.nl = reinterpret_cast<int *>(p + off); off += align16(sizeof(int) * R.S);
    w.lp = nullptr;
    w.loc = nullptr;
    w.q = nullptr;
    w.cen = reinterpret_cast<float4 *>(p + off); off += align16(sizeof(float4) * R.S);
    w.gb = reinterpret_cast<float4 *>(p + off); off += align16(sizeof(float4) * R.G);
    w.gA = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * R.G);
    w.cand = reinterpret_cast<int *>(p + off); off += align16(sizeof(int) * kWarp);
    w.cmask = reinterpret_cast<unsigned *>(p + off);
}

// FK of a chunk's ks states, all chains advancing together: first the ks x (L - 1)
// joint-local transforms of links 1.. spread over the lanes link-major (the lanes of one
// pass mostly share a joint type, so the type branches diverge little; link 0 is the
// identity and needs none), then the chains, one pose row a lane (below).  qv(k, i) is
// joint i of state k.  The arithmetic is warp_fk's (joint_local, mul_elem), so poses are
// bit-identical.
template <int K, typename QV>
__device__ inline void warp_fk_chunk_q(const SmemTables &t, int L, int ks, QV qv, float *locK, float *lpK, int lane) {
    for (int idx = lane; idx < ks * (L - 1); idx += kWarp) {
        const int i = 1 + idx / ks, k = idx - (i - 1) * ks;
        joint_local(t, i, qv(k, i), locK + 12 * (k * L + i));
    }
    __syncwarp();
    // Composition: lane 3 k + r (k < ks) owns row r of state k's poses and walks the
    // links in order.  The parent's row is the lane's own: in registers while the parent
    // is the previous link, else its own earlier store, so no lane waits on another.
    // Rows and joint-local transforms are 16-byte aligned (48-byte poses in a block
    // carved on 16 bytes) and move as float4.
    static_assert(3 * K <= kWarp, "one lane per pose row of every state of a chunk");
    const int kr = lane / 3, rr = lane - 3 * kr;
    if (lane < 3 * ks) {
        float4 *rowp = reinterpret_cast<float4 *>(lpK + kr * 12 * L) + rr;   // row rr of link 0
        float4 a = make_float4(rr == 0 ? 1.f : 0.f, rr == 1 ? 1.f : 0.f, rr == 2 ? 1.f : 0.f, 0.f);
        *rowp = a;
        const float4 *loc = reinterpret_cast<const float4 *>(locK + kr * 12 * L);
        for (int i = 1; i < L; ++i) {
            const int ty = t.type[i], par = t.parent[i];
            if (par != i - 1) a = rowp[3 * par];
            float4 o;
            if (ty == 1 || ty == 2 || ty == 5) {
                const float4 b0 = loc[3 * i], b1 = loc[3 * i + 1], b2 = loc[3 * i + 2];
                o.x = __fmaf_rn(a.z, b2.x, __fmaf_rn(a.y, b1.x, __fmul_rn(a.x, b0.x)));
                o.y = __fmaf_rn(a.z, b2.y, __fmaf_rn(a.y, b1.y, __fmul_rn(a.x, b0.y)));
                o.z = __fmaf_rn(a.z, b2.z, __fmaf_rn(a.y, b1.z, __fmul_rn(a.x, b0.z)));
                o.w = __fadd_rn(__fmaf_rn(a.z, b2.w, __fmaf_rn(a.y, b1.w, __fmul_rn(a.x, b0.w))), a.w);
            } else {
                o = make_float4(rr == 0 ? 1.f : 0.f, rr == 1 ? 1.f : 0.f, rr == 2 ? 1.f : 0.f, 0.f);
            }
            rowp[3 * i] = o;
            a = o;
        }
    }
    __syncwarp();
}

// FK of the chunk's ks states of one edge (state s = s0 + k from f towards t by d, the
// last state of the edge exactly t).
template <int K>
__device__ inline void warp_fk_chunk(const SmemTables &t, int L, int ks, const float *__restrict__ f,
                                     const float *__restrict__ to, const float *__restrict__ d, int s0, int n,
                                     float *locK, float *lpK, int lane) {
    warp_fk_chunk_q<K>(
        t, L, ks,
        [&](int k, int i) {
            const int s = s0 + k;
            return (s == n - 1) ? to[i] : __fmaf_rn(d[i], (float)s, f[i]);
        },
        locK, lpK, lane);
}

// Append this lane's obstacle (when mask != 0) to the candidate list; returns the new
// warp-uniform count (which may exceed the list, meaning overflow).
__device__ __forceinline__ int push_cand(const ChunkScratch &cs, int n, unsigned idx, unsigned mask, int lane) {
    const unsigned bal = __ballot_sync(kFull, mask != 0u);
    if (mask) {
        const int pos = n + __popc(bal & ((1u << lane) - 1u));
        if (pos < kChunkCands) { cs.cl[pos] = idx; cs.cm[pos] = mask; }
    }
    return n + __popc(bal);
}

// Groups (bit q) whose swept sphere touches the bounding sphere of run c0 + lane of an
// obstacle type with nruns runs; 0 for lanes past the last run.
__device__ __forceinline__ unsigned run_groups(const float4 *runs, int nruns, int c0, const ChunkScratch &cs, int G,
                                               int lane) {
    const int c = c0 + lane;
    unsigned gm = 0u;
    if (c < nruns) {
        const float4 b = runs[c];
        for (int q = 0; q < G; ++q) {
            const float4 gs = cs.sgb[q];
            const float rr = gs.w + b.w;
            if (sq3(gs.x - b.x, gs.y - b.y, gs.z - b.z) < rr * rr) gm |= 1u << q;
        }
    }
    return gm;
}

// xform_point for a link pose in the chunk's pose block, which is 16-byte aligned (the
// block starts on 16 bytes and every pose is 48 bytes): three float4 loads, the same
// arithmetic.
__device__ __forceinline__ float3 xform_point_a16(const float *T, float x, float y, float z) {
    const float4 *T4 = reinterpret_cast<const float4 *>(T);
    const float4 r0 = T4[0], r1 = T4[1], r2 = T4[2];
    float3 o;
    o.x = __fadd_rn(__fmaf_rn(r0.z, z, __fmaf_rn(r0.y, y, __fmul_rn(r0.x, x))), r0.w);
    o.y = __fadd_rn(__fmaf_rn(r1.z, z, __fmaf_rn(r1.y, y, __fmul_rn(r1.x, x))), r1.w);
    o.z = __fadd_rn(__fmaf_rn(r2.z, z, __fmaf_rn(r2.y, y, __fmul_rn(r2.x, x))), r2.w);
    return o;
}

// Exact tests of one state (link poses lp) against the chunk's candidates, then its
// self-collision pairs.  ns_end / nb_end / nc_end delimit the sphere / cuboid /
// cylinder candidates; `need` holds the groups any candidate or listed group pair
// involves (spheres of other groups cannot collide in this chunk and are not placed),
// and cs.nl lists their nn spheres, packed into the lanes' slots (about 3.4 of the 8
// groups of the benchmark arm are needed per state, so two slots of four hold them and
// the slots past the last sphere are skipped); npr group pairs are listed in cs.pl
// unless pairs_overflow.
template <int SPL, bool CNT>
__device__ inline bool chunk_state(const SmemTables &t, const DevRobot &R, const DevEnv &E, const WarpScratch &w,
                                   const ChunkScratch &cs, const float *lp, int ns_end, int nb_end, int nc_end,
                                   unsigned need, unsigned pneed, int npr, bool pairs_overflow, int nn, int lane,
                                   unsigned long long &fl) {
    constexpr bool count = CNT;   // executed-work accounting compiled in only when asked for
    float cx[SPL], cy[SPL], cz[SPL], cr[SPL], A[SPL];
    unsigned gbit[SPL];
    const int ms = (nn + kWarp - 1) / kWarp;   // slots holding a sphere on some lane
#pragma unroll
    for (int m = 0; m < SPL; ++m) {
        const int idx = lane + kWarp * m;
        const bool place = idx < nn;
        if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, place)) * 24;
        if (place) {
            const int k = cs.nl[idx];
            const float4 s = t.sph[k];
            const float3 p = xform_point_a16(lp + 12 * t.slink[k], s.x, s.y, s.z);
            cx[m] = p.x; cy[m] = p.y; cz[m] = p.z; cr[m] = s.w;
            gbit[m] = 1u << t.sgrp[k];
            if (pneed & gbit[m]) w.cen[k] = make_float4(p.x, p.y, p.z, s.w);   // only self pairs read it
        } else {
            cx[m] = kFar; cy[m] = kFar; cz[m] = kFar; cr[m] = 0.f;
            gbit[m] = 0u;
        }
        A[m] = __fmaf_rn(cz[m], cz[m], __fmaf_rn(cy[m], cy[m], __fmaf_rn(cx[m], cx[m], -cr[m] * cr[m])));
    }
    if (lane < R.G && ((pneed >> lane) & 1u)) {
        const float4 g = t.grp[lane];
        const float3 c = xform_point_a16(lp + 12 * t.glink[lane], g.x, g.y, g.z);
        w.gb[lane] = make_float4(c.x, c.y, c.z, g.w);
    }
    __syncwarp();
    bool hit = false;

    // --- obstacle spheres (expanded form, see warp_collide) ---
    const float4 *sx = t.env + E.ns + 5 * E.nb + 4 * E.nc;
    const float *snb = reinterpret_cast<const float *>(sx + E.ns);
    for (int i = 0; i < ns_end; ++i) {
        const unsigned o = cs.cl[i], cm = cs.cm[i];
        const float4 b = sx[o];
        const float nb = snb[o];
#pragma unroll
        for (int m = 0; m < SPL; ++m) {
            if (m >= ms) break;
            const float v = __fmaf_rn(cx[m], b.x, __fmaf_rn(cy[m], b.y, __fmaf_rn(cz[m], b.z, __fmaf_rn(cr[m], b.w, nb))));
            hit |= (cm & gbit[m]) && v > A[m];
            if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, (cm & gbit[m]) != 0u)) * kFlSphereX;
        }
    }
    if (ns_end > 0 && __any_sync(kFull, hit)) return true;

    // --- cuboids ---
    const float4 *bx = t.env + E.ns;
    for (int i = ns_end; i < nb_end; ++i) {
        const unsigned o = cs.cl[i], cm = cs.cm[i];
        const float4 r0 = bx[5 * o], r1 = bx[5 * o + 1], r2 = bx[5 * o + 2], mn = bx[5 * o + 3], mx = bx[5 * o + 4];
#pragma unroll
        for (int m = 0; m < SPL; ++m) {
            if (m >= ms) break;
            if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, (cm & gbit[m]) != 0u)) * kFlCuboid;
            if (cm & gbit[m]) {
                const float3 l = xform_rows(r0, r1, r2, cx[m], cy[m], cz[m]);
                const float dx = l.x - fminf(fmaxf(l.x, mn.x), mx.x);
                const float dy = l.y - fminf(fmaxf(l.y, mn.y), mx.y);
                const float dz = l.z - fminf(fmaxf(l.z, mn.z), mx.z);
                hit |= sq3(dx, dy, dz) < cr[m] * cr[m];
            }
        }
    }
    if (nb_end > ns_end && __any_sync(kFull, hit)) return true;

    // --- cylinders ---
    const float4 *cyl = t.env + E.ns + 5 * E.nb;
    for (int i = nb_end; i < nc_end; ++i) {
        const unsigned o = cs.cl[i], cm = cs.cm[i];
        const float4 r0 = cyl[4 * o], r1 = cyl[4 * o + 1], r2 = cyl[4 * o + 2], pr = cyl[4 * o + 3];
#pragma unroll
        for (int m = 0; m < SPL; ++m) {
            if (m >= ms) break;
            if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, (cm & gbit[m]) != 0u)) * kFlCylinder;
            if (cm & gbit[m]) {
                const float3 l = xform_rows(r0, r1, r2, cx[m], cy[m], cz[m]);
                const float dx = sqrtf(__fmaf_rn(l.y, l.y, __fmul_rn(l.x, l.x))) - pr.x;
                const float dz = fabsf(l.z) - pr.y;
                const float ox = dx > 0.f ? dx : 0.f, oz = dz > 0.f ? dz : 0.f;
                const float outside = sqrtf(__fmaf_rn(oz, oz, __fmul_rn(ox, ox)));
                const float inside = fminf(fmaxf(dx, dz), 0.f);
                hit |= cr[m] - (outside + inside) > 0.f;
            }
        }
    }
    if (nc_end > nb_end && __any_sync(kFull, hit)) return true;

    // --- self collision: listed group pairs whose per-state bounding spheres overlap ---
    const int nlist = pairs_overflow ? R.NPL : npr;
    for (int k0 = 0; k0 < nlist; k0 += kWarp) {
        const int k = k0 + lane;
        bool on = false;
        int p0 = 0, p1 = 0;
        int ga = 0, gb = 0;
        if (k < nlist) {
            const int4 lpr = t.lpair[pairs_overflow ? k : cs.pl[k]];
            const float4 a = w.gb[lpr.x], b = w.gb[lpr.y];
            const float rr = a.w + b.w;
            // (with pairs_overflow every enabled pair is walked; a group outside `need`
            // has no sphere placed this state, and its pairs cannot touch in this chunk)
            on = ((pneed >> lpr.x) & (pneed >> lpr.y) & 1u) && sq3(a.x - b.x, a.y - b.y, a.z - b.z) < rr * rr;
            ga = lpr.x;
            gb = lpr.y;
            p0 = lpr.z;
            p1 = lpr.w;
        }
        unsigned bal = __ballot_sync(kFull, on);
        if (count) fl += (unsigned long long)min(kWarp, nlist - k0) * kFlGroupPair;
        while (bal) {
            const int j = __ffs(bal) - 1;
            bal &= bal - 1u;
            const int q0 = __shfl_sync(kFull, p0, j), q1 = __shfl_sync(kFull, p1, j);
            const int xa = __shfl_sync(kFull, ga, j), xb = __shfl_sync(kFull, gb, j);
            const int a0 = t.gso[xa], na = t.gso[xa + 1] - a0, b0 = t.gso[xb], nb = t.gso[xb + 1] - b0;
            if (na <= kWarp && nb <= kWarp && q1 - q0 == na * nb) {
                // The range holds every (sphere of a, sphere of b) pair.  A sphere of a can
                // touch a sphere of b only if it touches b's bounding sphere (and the other
                // way round), so only pairs of such spheres are tested, with the pair
                // threshold (ri + rj)^2 rounded as the pair list's.  The spheres of a stay
                // in the registers of their lanes and are broadcast by shuffles.
                const float4 GA = w.gb[xa], GB = w.gb[xb];
                bool ia = false, ib = false;
                float4 cj = make_float4(kFar, kFar, kFar, 0.f), c = cj;
                // b's spheres against a's group sphere first: when none touches it, no
                // pair of this group pair can touch and a's spheres are not loaded
                if (lane < nb) {
                    cj = w.cen[t.gsl[b0 + lane]];
                    const float rr = cj.w + GA.w;
                    ib = sq3(cj.x - GA.x, cj.y - GA.y, cj.z - GA.z) < rr * rr;
                }
                const unsigned mb = __ballot_sync(kFull, ib);
                if (mb && lane < na) {
                    c = w.cen[t.gsl[a0 + lane]];
                    const float rr = c.w + GB.w;
                    ia = sq3(c.x - GB.x, c.y - GB.y, c.z - GB.z) < rr * rr;
                }
                unsigned ma = __ballot_sync(kFull, ia);
                if (count) fl += (unsigned long long)(nb + (mb ? na : 0) + __popc(ma) * __popc(mb)) * kFlSelf;
                while (ma) {
                    const int x = __ffs(ma) - 1;
                    ma &= ma - 1u;
                    const float4 ci = make_float4(__shfl_sync(kFull, c.x, x), __shfl_sync(kFull, c.y, x),
                                                  __shfl_sync(kFull, c.z, x), __shfl_sync(kFull, c.w, x));
                    if (ib) {
                        const float sr = __fadd_rn(ci.w, cj.w);
                        hit |= sq3(ci.x - cj.x, ci.y - cj.y, ci.z - cj.z) < __fmul_rn(sr, sr);
                    }
                }
            } else {
                if (count) fl += (unsigned long long)(q1 - q0) * kFlSelf;
                for (int p = q0 + lane; p < q1; p += kWarp) {
                    const unsigned ij = __ldg(R.pairs + p);
                    const float thr = __ldg(R.thr + p);
                    const float4 a = w.cen[ij & 0xffffu], b = w.cen[ij >> 16];
                    hit |= sq3(a.x - b.x, a.y - b.y, a.z - b.z) < thr;
                }
            }
            if (__any_sync(kFull, hit)) return true;
        }
    }
    return false;
}

// Per-state routine for a chunk whose candidates overflow the list; out of line, since
// it runs rarely and inlining it would crowd the instruction cache of the common path.
template <int SPL>
__device__ __noinline__ bool chunk_fallback(const SmemTables &t, const DevRobot &R, const DevEnv &E, WarpScratch w,
                                            const float *lp, int lane) {
    w.lp = const_cast<float *>(lp);
    return warp_collide_culled<SPL>(t, R, E, w, lane);
}

// States [s0, s1) of one edge (from f to t with per-state step d, n states in all).
// Returns the first colliding state, or -1 (also when another warp already recorded
// a hit below the state reached).
template <int SPL, int K, bool CNT>
__device__ inline int warp_edge_chunk(const SmemTables &t, const DevRobot &R, const DevEnv &E, const WarpScratch &w,
                                      const ChunkScratch &cs, int lane, const float *__restrict__ f,
                                      const float *__restrict__ to, const float *__restrict__ d, int s0, int s1,
                                      int n) {
    const int ks = s1 - s0;
    constexpr bool count = CNT;   // executed-work accounting compiled in only when asked for
    // FK and the group-centre transforms of every state; sphere placements are counted
    // where they happen
    unsigned long long fl = (unsigned long long)(R.base_flops - 24LL * R.S) * ks;

    // --- A: FK of every state, box of each group centre ---
    const bool gl = lane < R.G;
    const float4 g = gl ? t.grp[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    float lox = 3.0e38f, loy = 3.0e38f, loz = 3.0e38f, hix = -3.0e38f, hiy = -3.0e38f, hiz = -3.0e38f;
    warp_fk_chunk<K>(t, R.L, ks, f, to, d, s0, n, cs.locK, cs.lpK, lane);
    // group centres of every (state, group) pair, spread over the lanes, into the region
    // the joint-local transforms used (dead now; ks x G float4 fit in it since G <= L)
    float4 *gc = reinterpret_cast<float4 *>(cs.locK);
    for (int p = lane; p < ks * R.G; p += kWarp) {
        const int k = p / R.G, q = p - k * R.G;
        const float4 gq = t.grp[q];
        const float3 c = xform_point_a16(cs.lpK + k * 12 * R.L + 12 * t.glink[q], gq.x, gq.y, gq.z);
        gc[p] = make_float4(c.x, c.y, c.z, 0.f);
    }
    __syncwarp();
    if (gl) {
        for (int k = 0; k < ks; ++k) {
            const float4 c = gc[k * R.G + lane];
            lox = fminf(lox, c.x); loy = fminf(loy, c.y); loz = fminf(loz, c.z);
            hix = fmaxf(hix, c.x); hiy = fmaxf(hiy, c.y); hiz = fmaxf(hiz, c.z);
        }
    }
    __syncwarp();   // the swept spheres below overwrite the start of that region

    // --- B: swept group spheres ---
    if (gl) {
        const float cx = 0.5f * (lox + hix), cy = 0.5f * (loy + hiy), cz = 0.5f * (loz + hiz);
        const float hx = 0.5f * (hix - lox), hy = 0.5f * (hiy - loy), hz = 0.5f * (hiz - loz);
        const float rad = sqrtf(hx * hx + hy * hy + hz * hz) + g.w;
        cs.sgb[lane] = make_float4(cx, cy, cz, rad);
        cs.sgA[lane] = __fmaf_rn(cz, cz, __fmaf_rn(cy, cy, __fmaf_rn(cx, cx, -rad * rad)));
    }
    __syncwarp();

    // --- C: broad phase of the chunk, run spheres first ---
    // The bounding spheres of all runs (sphere runs, then box runs, then cylinder runs)
    // are tested in one pass, lane j taking run c0 + j against every swept group sphere;
    // only runs some group touches are visited, in run order (so the candidates come out
    // grouped by obstacle type), and their obstacles are tested only against the groups
    // that touched the run.
    int nc = 0, nsph = 0, nbox = 0;
    unsigned need = 0u;
    const float4 *sx = t.env + E.ns + 5 * E.nb + 4 * E.nc;
    const float *snb = reinterpret_cast<const float *>(sx + E.ns);
    const float4 *bx = t.env + E.ns;
    const float4 *cyl = t.env + E.ns + 5 * E.nb;
    const int nrs = env_clusters(E.ns), nrb = env_clusters(E.nb), nrun = nrs + nrb + env_clusters(E.nc);
    const float4 *runs_w = t.env + env_cluster_base(E.ns, E.nb, E.nc);
#pragma unroll 1
    for (int c0 = 0; c0 < nrun; c0 += kWarp) {
        const unsigned gmc = run_groups(runs_w, nrun, c0, cs, R.G, lane);
        unsigned runs = __ballot_sync(kFull, gmc != 0u);
        if (count) fl += (unsigned long long)min(kWarp, nrun - c0) * R.G * kFlGroupPair;
        while (runs) {
            const int j = __ffs(runs) - 1;
            runs &= runs - 1u;
            const unsigned gm = __shfl_sync(kFull, gmc, j);
            const int c = c0 + j;
            unsigned mask = 0u;
            int o;
            if (c < nrs) {   // obstacle spheres (expanded form, see warp_collide)
                o = c * kWarp + lane;
                if (o < E.ns) {
                    const float4 b = sx[o];
                    const float nb = snb[o];
                    for (unsigned m = gm; m; m &= m - 1u) {
                        const int q = __ffs(m) - 1;
                        const float4 gs = cs.sgb[q];
                        const float v = __fmaf_rn(gs.x, b.x, __fmaf_rn(gs.y, b.y, __fmaf_rn(gs.z, b.z, __fmaf_rn(gs.w, b.w, nb))));
                        if (v > cs.sgA[q]) mask |= 1u << q;
                    }
                }
                if (count) fl += (unsigned long long)min(kWarp, E.ns - c * kWarp) * __popc(gm) * kFlSphereX;
            } else if (c < nrs + nrb) {   // cuboids
                o = (c - nrs) * kWarp + lane;
                if (o < E.nb) {
                    const float4 r0 = bx[5 * o], r1 = bx[5 * o + 1], r2 = bx[5 * o + 2], mn = bx[5 * o + 3], mx = bx[5 * o + 4];
                    for (unsigned m = gm; m; m &= m - 1u) {
                        const int q = __ffs(m) - 1;
                        const float4 gs = cs.sgb[q];
                        const float3 l = xform_rows(r0, r1, r2, gs.x, gs.y, gs.z);
                        const float dx = l.x - fminf(fmaxf(l.x, mn.x), mx.x);
                        const float dy = l.y - fminf(fmaxf(l.y, mn.y), mx.y);
                        const float dz = l.z - fminf(fmaxf(l.z, mn.z), mx.z);
                        if (sq3(dx, dy, dz) < gs.w * gs.w) mask |= 1u << q;
                    }
                }
                if (count) fl += (unsigned long long)min(kWarp, E.nb - (c - nrs) * kWarp) * __popc(gm) * kFlCuboid;
            } else {   // cylinders
                o = (c - nrs - nrb) * kWarp + lane;
                if (o < E.nc) {
                    const float4 r0 = cyl[4 * o], r1 = cyl[4 * o + 1], r2 = cyl[4 * o + 2], pr = cyl[4 * o + 3];
                    for (unsigned m = gm; m; m &= m - 1u) {
                        const int q = __ffs(m) - 1;
                        const float4 gs = cs.sgb[q];
                        const float3 l = xform_rows(r0, r1, r2, gs.x, gs.y, gs.z);
                        const float dx = sqrtf(__fmaf_rn(l.y, l.y, __fmul_rn(l.x, l.x))) - pr.x;
                        const float dz = fabsf(l.z) - pr.y;
                        const float ox = dx > 0.f ? dx : 0.f, oz = dz > 0.f ? dz : 0.f;
                        const float sdf = sqrtf(__fmaf_rn(oz, oz, __fmul_rn(ox, ox))) + fminf(fmaxf(dx, dz), 0.f);
                        if (gs.w - sdf > 0.f) mask |= 1u << q;
                    }
                }
                if (count) fl += (unsigned long long)min(kWarp, E.nc - (c - nrs - nrb) * kWarp) * __popc(gm) * kFlCylinder;
            }
            const int before = nc;
            nc = push_cand(cs, nc, (unsigned)o, mask, lane);
            need |= mask;
            if (c < nrs) nsph += nc - before;
            else if (c < nrs + nrb) nbox += nc - before;
        }
    }
    const int ns_end = nsph, nb_end = nsph + nbox;
    // enabled group pairs whose swept spheres overlap
    int npr = 0;
    unsigned pneed = 0u;
    for (int k0 = 0; k0 < R.NPL; k0 += kWarp) {
        const int k = k0 + lane;
        bool on = false;
        if (k < R.NPL) {
            const int4 lpr = t.lpair[k];
            const float4 a = cs.sgb[lpr.x], b = cs.sgb[lpr.y];
            const float rr = a.w + b.w;
            on = sq3(a.x - b.x, a.y - b.y, a.z - b.z) < rr * rr;
            if (on) pneed |= (1u << lpr.x) | (1u << lpr.y);
        }
        const unsigned bal = __ballot_sync(kFull, on);
        if (on) {
            const int pos = npr + __popc(bal & ((1u << lane) - 1u));
            if (pos < kChunkPairs) cs.pl[pos] = k;
        }
        npr += __popc(bal);
        if (count) fl += (unsigned long long)min(kWarp, R.NPL - k0) * kFlGroupPair;
    }
    pneed = __reduce_or_sync(kFull, pneed);
    need = __reduce_or_sync(kFull, need) | pneed;
    __syncwarp();
    const bool overflow = nc > kChunkCands;
    const bool pairs_overflow = npr > kChunkPairs;

    // --- D: states in order ---
    int found = -1;
    const int kend = (need == 0u && !overflow) ? 0 : ks;   // nothing near any state: all free
    // the spheres of the needed groups, packed, so that the per-state slots hold only them
    int nn = 0;
    if (kend > 0 && !overflow) {
        for (int k0 = 0; k0 < R.S; k0 += kWarp) {
            const int k = k0 + lane;
            const bool in = k < R.S && ((need >> t.sgrp[k]) & 1u);
            const unsigned bal = __ballot_sync(kFull, in);
            if (in) cs.nl[nn + __popc(bal & ((1u << lane) - 1u))] = k;
            nn += __popc(bal);
        }
        __syncwarp();
    }
    for (int k = 0; k < kend; ++k) {
        const int s = s0 + k;
        const float *lp = cs.lpK + k * 12 * R.L;
        bool hit;
        if (overflow) {
            hit = chunk_fallback<SPL>(t, R, E, w, lp, lane);
        } else {
            hit = chunk_state<SPL, CNT>(t, R, E, w, cs, lp, ns_end, nb_end, nc, need, pneed, npr, pairs_overflow, nn,
                                        lane, fl);
        }
        __syncwarp();
        if (hit) {
            found = s;
            break;
        }
    }
    if (count && lane == 0) {
        atomicAdd(R.work, fl);
        atomicAdd(R.work + 1, (unsigned long long)ks);
    }
    return found;
}

}  // namespace gbmp
