// hrt_trace_w4.cuh -- the persistent diffuse trace over compressed 4-wide nodes for scenes
// without voxels, laid out for occupancy.
//
// The trace is bound by the latency of node fetches (L1/L2 hits) and by issue slots, not by
// DRAM.  More resident warps hide more of that latency, so this kernel keeps only the state
// of the node loop in registers -- the ray origin premultiplied by the inverse direction
// (ooi), the inverse direction, best distance, current node, two postponed leaves, stack
// pointer and visit budget -- and moves the rest of each lane's state to shared memory, where
// it is touched only when a ray starts, reaches a leaf or ends: the origin, the direction and
// the watertight-test set-up (kx, ky, kz, Sx, Sy, Sz), the best hit so far, the origin
// primitive and face, the wrap count, the running-sum key and sums.
// A node visit is kept short because the kernel is issue-bound: two 256-bit node loads, each
// slab offset in one fused multiply-add from ooi (node4_offset_ooi), the nearest hit child
// found by a three-comparator tournament (node4_nearest) and entered, the other hit children
// pushed without a branch between the hit and no-hit cases, pops with no empty-stack test (a
// sentinel at the bottom of the stack), leaves postponed two per lane, and the loop left only
// when fewer than P.refill lanes remain; ray ids are split into face, primitive, ray and
// stratum by multiplication (FastDiv).
// The traversal stack keeps SD entries per lane in shared memory (indexed [entry][lane], so
// the 32 lanes of a warp always hit 32 different banks) over a local overflow array, in one
// of two layouts.  RingStack: the top SD entries in a ring, entries deeper than SD below the
// top moved to local memory on push and brought back on pop.  LinStack (LIN): the bottom SD
// entries in shared memory, deeper ones in local memory, and a visit whose pushes all stay
// below SD writes them with no overflow test.  Local memory is touched only by rays whose
// stack is deeper than SD.  On the 1 M-triangle orchard LinStack with SD = 16 is the faster
// (180 against 184 ms per diffuse launch for the ring at SD = 16, 186-189 at SD = 8).
//
// Hits equal those of trace_bvh / k_diffuse_ps: the same node and primitive tests, the same
// tie rule (closest, then smaller original index); only the order of work differs.
#pragma once
#include <type_traits>

#include "hrt_trace.cuh"

namespace hrt {

namespace {

template <int SD, int BLOCK>
struct RingStack {
    static_assert((SD & (SD - 1)) == 0 && SD >= 2, "shared stack depth must be a power of two");
    int32_t (*ring)[BLOCK];   // [SD][BLOCK] in shared memory
    int tid;
    int32_t spill[kStack4];   // local memory, entries below the top SD
    __device__ __forceinline__ void push(int sp, int32_t v) {
        const int slot = sp & (SD - 1);
        if (sp >= SD) spill[sp - SD] = ring[slot][tid];
        ring[slot][tid] = v;
    }
    // value of entry sp (the entry just below the old top), restoring the ring window
    __device__ __forceinline__ int32_t pop(int sp) {
        const int slot = sp & (SD - 1);
        const int32_t v = ring[slot][tid];
        if (sp >= SD) ring[slot][tid] = spill[sp - SD];
        return v;
    }
};

// The bottom SD entries in shared memory ([entry][lane]), deeper ones in local memory (the
// kernel keeps a sentinel in entry 0, so SD - 1 of them hold nodes).
template <int SD, int BLOCK>
struct LinStack {
    int32_t (*ring)[BLOCK];   // [SD][BLOCK] in shared memory (not a ring: entry i at row i)
    int tid;
    int32_t spill[kStack4];
    __device__ __forceinline__ void push(int sp, int32_t v) {
        if (sp < SD) ring[sp][tid] = v;
        else spill[sp - SD] = v;
    }
    __device__ __forceinline__ int32_t pop(int sp) { return sp < SD ? ring[sp][tid] : spill[sp - SD]; }
};

// BLOCK: threads per block; MINB: resident blocks per SM the register allocation must allow.
// SD: stack entries per lane in shared memory (a power of two).  KB: ray-id batch -- a warp
// takes 32 x KB consecutive ray ids from the global counter at a time and hands them to its
// idle lanes from shared memory (KB = 1: every refill takes exactly the idle lanes' count).
// MULTI (recording mode only): the launch traces several scenes -- P.slots[0..P.nslots) each
// give a scene, a primitive chunk, ray counts, seed, pass and hit buffer, with consecutive
// ranges of the launch's ray ids (id_begin) -- so one persistent launch covers the pass of
// every scene of a multi-scene sweep.  LIN: the LinStack layout, else RingStack.
template <int NB, bool RECORD, bool STATS, int MINB, int SD, int BLOCK, int KB, bool MULTI = false, bool LIN = false>
__global__ void __launch_bounds__(BLOCK, MINB) k_diffuse_w4(const DiffuseParams P) {
    static_assert(!MULTI || (RECORD && !STATS), "multi-scene launches record hits only");
    __shared__ double s_sum[RECORD ? 1 : NB][BLOCK];            // running sums of the lane's origin
    __shared__ float s_ray[9][BLOCK];                            // d.xyz, Sx, Sy, Sz, o.xyz
    __shared__ uint32_t s_lane[5][BLOCK];                        // see the L_* slots below
    __shared__ int32_t s_stack[SD][BLOCK];
    __shared__ unsigned long long s_rid[RECORD ? BLOCK : 1];     // record: hit-buffer index
    __shared__ unsigned long long s_chunk[2][KB > 1 ? BLOCK / 32 : 1];  // per warp: next id, end
    __shared__ SceneSlot s_slot[MULTI ? kMaxSlots : 1];          // multi-scene: the launch's scenes
    __shared__ unsigned long long s_srays[MULTI ? kMaxSlots : 1];  // multi-scene: rays per scene
    constexpr int L_AXES = 0;  // kx | ky << 2 | kz << 4 | face << 6 | wraps << 8
    constexpr int L_P = 1;     // origin primitive
    constexpr int L_HIT = 2;   // best hit so far: prim << 1 | face, or kMissCode
    constexpr int L_KEY = 3;   // running-sum key 2p + face, or 0xFFFFFFFF
    constexpr int L_TAKEN = 4; // rays taken (lane budget)
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    // count x R x faces < 2^31: the host splits larger passes into primitive chunks
    const uint32_t per_face = P.count * R;
    const int nf = ((P.faces & 1) ? 1 : 0) + ((P.faces & 2) ? 1 : 0);
    const unsigned long long total = MULTI ? P.multi_total : (unsigned long long)per_face * (unsigned long long)nf;
    int lslot = 0;  // multi-scene: the scene slot of the lane's ray
    // single-scene launches decode ray ids (< 2^31, the host plans chunks) by multiplication:
    // 165.0 against 168.0 ms per diffuse launch of the 1 M-triangle orchard
    const FastDiv fd_face = make_fastdiv(per_face ? per_face : 1u), fd_r = make_fastdiv(R ? R : 1u),
                  fd_x = make_fastdiv(P.dimx > 0 ? (uint32_t)P.dimx : 1u);
    // the scene of the lane's current ray
#define SC (MULTI ? s_slot[lslot].sc : P.sc)
    if (MULTI) {
        const int words = P.nslots * (int)(sizeof(SceneSlot) / sizeof(uint32_t));
        const uint32_t *src = reinterpret_cast<const uint32_t *>(P.slots);
        uint32_t *dst = reinterpret_cast<uint32_t *>(s_slot);
        for (int i = tid; i < words; i += BLOCK) dst[i] = src[i];
        for (int i = tid; i < P.nslots; i += BLOCK) s_srays[i] = 0ull;
        __syncthreads();
    }

    typename std::conditional<LIN, LinStack<SD, BLOCK>, RingStack<SD, BLOCK>>::type stk;
    stk.ring = s_stack;
    stk.tid = tid;
    uint32_t nvis = 0, ntest = 0;  // statistics builds only
    uint32_t nrays = 0;
    bool live = false, exhausted = false;
    f3 ooi = mk(0.f, 0.f, 0.f), inv = ooi;
    float best = 1e38f;
    int32_t cur = kSentinel, leaf = 0, leaf2 = 0;  // current node, up to two postponed leaves
    // LIN: entry 0 of the shared stack holds kSentinel for good and a ray starts with sp = 1, so a
    // pop needs no empty-stack test: popping the sentinel ends the ray's traversal (168.7 against
    // 173.2 ms per diffuse launch of the 1 M-triangle orchard)
    constexpr int kSp0 = LIN ? 1 : 0;
    if (kSp0) s_stack[0][tid] = kSentinel;
    int sp = kSp0;
    uint32_t budget = 0;
    if (!RECORD) {
#pragma unroll
        for (int j = 0; j < NB; ++j) s_sum[j][tid] = 0.0;
    }
    s_lane[L_KEY][tid] = 0xFFFFFFFFu;
    s_lane[L_TAKEN][tid] = 0u;
    // a lane budget retires lanes without drawing ids, so a warp could leave ids of its
    // batch untraced: batched fetch only without one
    const bool batched = KB > 1 && P.lane_budget == 0;
    if (KB > 1 && lane == 0) {
        s_chunk[0][tid >> 5] = 0ull;
        s_chunk[1][tid >> 5] = 0ull;
    }
    __syncwarp();
#define POP() (kSp0 ? stk.pop(--sp) : (sp > 0 ? stk.pop(--sp) : kSentinel))

    for (;;) {
        // ---- refill lanes without a ray (warp-vote compaction of the fetch)
        if (!live && P.lane_budget && s_lane[L_TAKEN][tid] >= P.lane_budget) exhausted = true;
        const bool need = !live && !exhausted;
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            const unsigned rank = __popc(m & ((1u << lane) - 1u));
            unsigned long long id;
            if (!batched) {
                unsigned long long base = 0;
                if (lane == leader) base = atomicAdd(P.fetch, (unsigned long long)__popc(m));
                base = __shfl_sync(0xffffffffu, base, leader);
                id = base + rank;
            } else {
                // ids are handed out in increasing order, so every id below the end of the
                // range is drawn before any lane of the warp draws one past it
                const int w = tid >> 5;
                const unsigned nneed = __popc(m);
                const unsigned long long next = s_chunk[0][w], left = s_chunk[1][w] - next;
                unsigned long long nb = 0;
                if (left < nneed) {
                    if (lane == leader) nb = atomicAdd(P.fetch, (unsigned long long)(32 * KB));
                    nb = __shfl_sync(0xffffffffu, nb, leader);
                }
                id = rank < left ? next + rank : nb + (rank - left);
                __syncwarp();
                if (lane == leader) {
                    if (left < nneed) {
                        s_chunk[0][w] = nb + (nneed - left);
                        s_chunk[1][w] = nb + 32ull * KB;
                    } else {
                        s_chunk[0][w] = next + nneed;
                    }
                }
                __syncwarp();
            }
            if (need) {
                if (id >= total) {
                    exhausted = true;
                } else {
                    s_lane[L_TAKEN][tid] += 1u;
                    unsigned long long lid = id;
                    uint32_t Rk = R, pfk = per_face, offk = P.offset, seedk = P.seed, passk = P.pass;
                    int dxk = P.dimx, dyk = P.dimy;
                    if (MULTI) {  // the slot whose id range holds id (ranges are consecutive)
                        int k = 0;
                        while (k + 1 < P.nslots && id >= s_slot[k + 1].id_begin) ++k;
                        lslot = k;
                        const SceneSlot &S = s_slot[k];
                        lid = id - S.id_begin;
                        dxk = S.dimx;
                        dyk = S.dimy;
                        Rk = (uint32_t)(dxk * dyk);
                        pfk = S.count * Rk;
                        offk = S.offset;
                        seedk = S.seed;
                        passk = S.pass;
                    }
                    const TraceScene &sc = SC;
                    uint32_t fi, rem;
                    if (!MULTI) {
                        fi = fast_div((uint32_t)lid, fd_face);
                        rem = (uint32_t)lid - fi * pfk;
                    } else {
                        fi = (uint32_t)(lid / pfk);
                        rem = (uint32_t)(lid - (unsigned long long)fi * pfk);
                    }
                    const int face = (nf == 2) ? (fi == 0 ? 1 : 0) : ((P.faces & 1) ? 1 : 0);
                    uint32_t p, r, ti, pi;
                    if (!MULTI) {
                        const uint32_t q = fast_div(rem, fd_r);
                        p = offk + q;
                        r = rem - q * Rk;
                        pi = fast_div(r, fd_x);
                        ti = r - pi * (uint32_t)dxk;
                    } else {
                        p = offk + rem / Rk;
                        r = rem % Rk;
                        ti = r % (uint32_t)dxk;
                        pi = r / (uint32_t)dxk;
                    }
                    if (RECORD) s_rid[tid] = ((unsigned long long)fi * (unsigned long long)sc.n + p) * Rk + r;
                    const int ts = sc.twosided[p];
                    const bool skip = (face == 1 && ts == 3) || (face == 0 && ts != 1);
                    if (!skip) {
                        float4 g[4];
                        load_rgen(sc, p, g);
                        const uint32_t type = __float_as_uint(g[0].w);
                        f3 o, d;
                        diffuse_ray_cell<false>(g, type, r, p, face, (int)ti, (int)pi, dxk, dyk, seedk, passk, &o, &d,
                                                sc.masks);
                        const WT w = wt_setup(d);
                        s_ray[0][tid] = d.x;
                        s_ray[1][tid] = d.y;
                        s_ray[2][tid] = d.z;
                        s_ray[3][tid] = w.Sx;
                        s_ray[4][tid] = w.Sy;
                        s_ray[5][tid] = w.Sz;
                        s_ray[6][tid] = o.x;
                        s_ray[7][tid] = o.y;
                        s_ray[8][tid] = o.z;
                        s_lane[L_AXES][tid] = (uint32_t)(w.kx | (w.ky << 2) | (w.kz << 4) | (face << 6));
                        s_lane[L_P][tid] = p;
                        s_lane[L_HIT][tid] = kMissCode;
                        inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
                        ooi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
                        best = 1e38f;
                        cur = (sc.n > 0) ? 0 : kSentinel;
                        leaf = 0;
                        leaf2 = 0;
                        sp = kSp0;
                        budget = sc.visit_budget;
                        live = true;
                        if (MULTI) atomicAdd(&s_srays[lslot], 1ull);
                        else ++nrays;
                    }
                }
            }
        }
        // A lane may be idle because its id was skipped by the face rule; only when every
        // lane has run past the end of the id range is the warp done.
        if (__all_sync(0xffffffffu, exhausted && !live)) break;
        if (!live) continue;

        // ---- internal nodes; up to two leaves per lane are postponed to the primitive tests below
        const TraceScene &sc = SC;
        const uint32_t n4 = (uint32_t)sc.n4;
        // cur is an internal node: 0 <= cur < kSentinel in one unsigned compare (leaves are
        // negative; indices at or above n4 fail the bounds test inside)
        while ((uint32_t)cur < (uint32_t)kSentinel) {
            // both tests evaluated (no short-circuit branch), then the visit is counted
            if (((uint32_t)cur >= n4) | (budget == 0u)) {
                raise(sc.status, (uint32_t)cur >= n4 ? ERR_BOUNDS : ERR_BUDGET);
                cur = kSentinel;
                leaf = 0;
                leaf2 = 0;
                sp = kSp0;
                break;
            }
            --budget;
            if (STATS) ++nvis;
            float4 q0, q1, q2, q3;
            load_node64(sc.nodes4, cur, q0, q1, q2, q3);
            float tk[4];
            int32_t ck[4];  // every slot's reference: a child is hit when its tk < INFINITY
            node4_children<false>(q0, q1, q2, q3, node4_offset_ooi(q0, ooi, inv), inv, 1e-4f, best, tk, ck);
            node4_nearest(tk, ck);
            if (LIN) {
                // hit children other than the nearest pushed (predicated: a visit that hits
                // nothing pushes nothing), then the nearest entered or, with no hit, the top of
                // the stack taken -- no branch between the two cases
                const bool any = tk[0] < INFINITY;
                if (sp + 3 <= SD) {  // the whole push in shared memory
#pragma unroll
                    for (int k = 3; k >= 1; --k)
                        if (tk[k] < INFINITY) s_stack[sp++][tid] = ck[k];
                } else {
                    if (any && sp + 3 > SD + kStack4) {
                        raise(sc.status, ERR_STACK);
                        cur = kSentinel;
                        leaf = 0;
                        leaf2 = 0;
                        sp = kSp0;
                        break;
                    }
#pragma unroll
                    for (int k = 3; k >= 1; --k)
                        if (tk[k] < INFINITY) stk.push(sp++, ck[k]);
                }
                int32_t nxt = ck[0];
                if (!any) nxt = POP();
                cur = nxt;
            } else if (!(tk[0] < INFINITY)) {
                cur = POP();
            } else {
                if (sp + 3 > SD + kStack4) {
                    raise(sc.status, ERR_STACK);
                    cur = kSentinel;
                    leaf = 0;
                    leaf2 = 0;
                    sp = kSp0;
                    break;
                }
#pragma unroll
                for (int k = 3; k >= 1; --k)
                    if (tk[k] < INFINITY) stk.push(sp++, ck[k]);
                cur = ck[0];
            }
            // a leaf is postponed while one of the two slots is free; a lane with both full stops
            // at its third leaf.  The warp leaves the loop only when fewer than P.refill lanes
            // remain in it (no vote on the leaves): 162.7 against 167.4 ms per diffuse launch of
            // the 1 M-triangle orchard with one slot and a leave-when-all-have-a-leaf vote
            if (cur < 0 && leaf2 == 0) {
                if (leaf == 0) leaf = cur;
                else leaf2 = cur;
                cur = POP();
            }
            if (__popc(__activemask()) < P.refill) break;
        }
        // ---- primitive tests (origin, direction and watertight set-up come back from shared memory)
        if (leaf != 0) {
            const f3 o = mk(s_ray[6][tid], s_ray[7][tid], s_ray[8][tid]);
            const f3 d = mk(s_ray[0][tid], s_ray[1][tid], s_ray[2][tid]);
            const uint32_t ax = s_lane[L_AXES][tid];
            WT w;
            w.kx = (int)(ax & 3u);
            w.ky = (int)((ax >> 2) & 3u);
            w.kz = (int)((ax >> 4) & 3u);
            w.Sx = s_ray[3][tid];
            w.Sy = s_ray[4][tid];
            w.Sz = s_ray[5][tid];
            uint32_t bcode = s_lane[L_HIT][tid];
            const VoxKey vk{0u, 0u, 0u, 0u, 0u};  // no voxels in this kernel's scenes
            while (leaf != 0) {
                const uint32_t slot = (uint32_t)(~leaf);
                if (STATS) ++ntest;
                if (slot < (uint32_t)sc.n) {
                    float t;
                    int fc;
                    uint32_t orig;
                    if (rec_hit<false>(sc.rec, slot, w, o, d, inv, 1e-4f, best, vk, &t, &fc, &orig, sc.masks)) {
                        if (bcode == kMissCode || t < best || (t == best && orig < (bcode >> 1))) {
                            best = t;
                            bcode = (orig << 1) | (uint32_t)fc;
                        }
                    }
                } else {
                    raise(sc.status, ERR_BOUNDS);
                }
                leaf = leaf2;
                leaf2 = 0;
                if (leaf == 0 && cur < 0) {
                    leaf = cur;
                    cur = POP();
                }
            }
            s_lane[L_HIT][tid] = bcode;
        }
        if (cur != kSentinel || leaf != 0) continue;  // traversal of this ray goes on next round

        // ---- periodic walls: wrap and restart, or finish the ray
        const uint32_t bcode = s_lane[L_HIT][tid];
        bool lost = false;
        if (sc.nbbox > 0) {
            const f3 o = mk(s_ray[6][tid], s_ray[7][tid], s_ray[8][tid]);
            const f3 d = mk(s_ray[0][tid], s_ray[1][tid], s_ray[2][tid]);
            float tb;
            int which = -1;
            if (wall_closest(sc, o, d, 1e-4f, (bcode != kMissCode) ? best : 1e38f, &tb, &which) &&
                (bcode == kMissCode || tb < best)) {
                const uint32_t ax = s_lane[L_AXES][tid];
                const uint32_t wraps = ax >> 8;
                if (wraps >= 9) {
                    lost = true;
                } else {
                    f3 hp = add(o, scl(d, tb));
                    if ((sc.periodic_x == 1.f) && which < 2) {
                        const float width = sc.bbox[4].x - sc.bbox[0].x;
                        hp.x = hp.x + ((which == 0) ? width : -width);
                    } else {
                        const int yb = (sc.periodic_x == 1.f) ? 2 : 0;
                        const float width = sc.bbox[4 * (yb + 1)].y - sc.bbox[4 * yb].y;
                        hp.y = hp.y + ((which == yb) ? width : -width);
                    }
                    s_ray[6][tid] = hp.x;
                    s_ray[7][tid] = hp.y;
                    s_ray[8][tid] = hp.z;
                    ooi = mk(hp.x * inv.x, hp.y * inv.y, hp.z * inv.z);
                    best = 1e38f;
                    s_lane[L_HIT][tid] = kMissCode;
                    s_lane[L_AXES][tid] = (ax & 0xFFu) | ((wraps + 1u) << 8);
                    cur = 0;
                    sp = kSp0;
                    budget = sc.visit_budget;
                    continue;
                }
            }
        }
        // ---- value of the finished ray, added to the lane's running sum
        live = false;
        if (RECORD) {
            (MULTI ? s_slot[lslot].hits : P.hits)[s_rid[tid]] = lost ? kLostCode : bcode;
            continue;
        }
        if (lost) continue;
        const uint32_t face = (s_lane[L_AXES][tid] >> 6) & 1u;
        const uint32_t key = 2u * s_lane[L_P][tid] + face;
        const uint32_t akey = s_lane[L_KEY][tid];
        if (key != akey) {
            if (akey != 0xFFFFFFFFu) {
                double *dst = ((akey & 1u) ? P.Gt : P.Gb) + (size_t)(akey >> 1) * P.Bl;
#pragma unroll
                for (int j = 0; j < NB; ++j)
                    if (j < P.Bc && s_sum[j][tid] != 0.0) atomicAdd(dst + j, s_sum[j][tid]);
            }
            s_lane[L_KEY][tid] = key;
#pragma unroll
            for (int j = 0; j < NB; ++j) s_sum[j][tid] = 0.0;
        }
        if (bcode != kMissCode) {
            const float *src = ((bcode & 1u) ? P.otop : P.obot) + (size_t)(bcode >> 1) * P.Bl;
#pragma unroll
            for (int j = 0; j < NB; ++j)
                if (j < P.Bc) s_sum[j][tid] += (double)__ldg(src + j);
        } else {
            const f3 d = mk(s_ray[0][tid], s_ray[1][tid], s_ray[2][tid]);
#pragma unroll
            for (int j = 0; j < NB; ++j)
                if (j < P.Bc) {
                    const float fl = P.sky.flux[j];
                    if (fl > 0.f) s_sum[j][tid] += sky_fd(d, P.sky, j) * (double)fl;
                }
        }
    }
    if (!RECORD) {
        const uint32_t akey = s_lane[L_KEY][tid];
        if (akey != 0xFFFFFFFFu) {
            double *dst = ((akey & 1u) ? P.Gt : P.Gb) + (size_t)(akey >> 1) * P.Bl;
#pragma unroll
            for (int j = 0; j < NB; ++j)
                if (j < P.Bc && s_sum[j][tid] != 0.0) atomicAdd(dst + j, s_sum[j][tid]);
        }
    }
    if (MULTI) {  // every warp of the block is past its loop: count the rays per scene
        __syncthreads();
        for (int i = tid; i < P.nslots; i += BLOCK)
            if (s_srays[i] && s_slot[i].sc.rays) atomicAdd(s_slot[i].sc.rays, s_srays[i]);
    } else {
        if (P.sc.rays && nrays) atomicAdd(P.sc.rays, (unsigned long long)nrays);
    }
    if (STATS && P.sc.visits) {
        atomicAdd(P.sc.visits, (unsigned long long)nvis);
        atomicAdd(P.sc.visits + 1, (unsigned long long)ntest);
    }
#undef POP
#undef SC
}

}  // namespace

}  // namespace hrt
