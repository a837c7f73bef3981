// avbd_events.cu — contact and trigger events of the AVBD step.
//
// Reference: crates/physics/src/avbd/mod.rs:1606-1669 (emit_events: trigger
// enter/exit, contact begin/end from the deepest point of each pair against
// CONTACT_BEGIN_SLOP, hits above CONTACT_HIT_THRESHOLD) and :935-960 /
// :1126-1136 (a swept time-of-impact clamp is a hit unless the substep
// already reported one for that pair).
//
// Device layout.  The previous touch set is kept per body b (the higher
// handle of each pair) as a CSR of the lower handles in ascending order, in
// two alternating buffers.  At an emitting substep one thread per body b
// merges its touching B-side pairs (the B-side list is in ascending A
// order) with that list: Begin / End / Hit counts, exclusive scans over the
// bodies give every event its slot, and a second pass writes them.  Events
// of one substep therefore come out ordered by (body_b, body_a) — the same
// set as the reference's (body_a, body_b) order.  Trigger overlaps are few:
// discovery appends them, one CTA sorts them and diffs them against the
// previous set.
#include "avbd_common.cuh"

namespace avbd {

constexpr float CONTACT_BEGIN_SLOP = 0.005f;   // trigger.rs:68
constexpr float CONTACT_HIT_THRESHOLD = 1.0f;  // trigger.rs:63

// deepest point and approach of every pair (mod.rs:1624-1642)
__global__ void k_ev_touch(DW w) {
    if (aborted_solve(w)) return;
    const uint32_t n = n_pairs(w);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint2 ab = w.p_ab[p];
        float4 n4 = w.p_n[p];
        V3 nn = ld3(n4);
        V3 pa0 = ld3(w.pos[ab.x]), pb0 = ld3(w.pos[ab.y]);
        Q qa = ldq(w.rot[ab.x]), qb = ldq(w.rot[ab.y]);
        float deepest = 0.0f;
        V3 witness = (pa0 + pb0) * HALF;
        uint32_t np = w.p_np[p];
        for (uint32_t k = 0; k < np; k++) {
            uint32_t q = p * MAX_PTS + k;
            V3 pa = pa0 + qrot(qa, ld3(w.q_ra[q]));
            V3 pb = pb0 + qrot(qb, ld3(w.q_rb[q]));
            float gap = dot(nn, pa - pb);
            if (-gap > deepest) {
                deepest = -gap;
                witness = pa;
            }
        }
        float approach = -dot(ld3(w.pre_vel[ab.x]) - ld3(w.pre_vel[ab.y]), nn);
        w.t_flag[p] = deepest > CONTACT_BEGIN_SLOP ? 1u : 0u;
        w.t_wit[p] = st3(witness, approach);
    }
}

// Is (a, b) in the touch set whose CSR is (off, keys)?
static __device__ __forceinline__ bool in_touch_set(const uint32_t* off, const uint32_t* keys, uint32_t a,
                                                    uint32_t b) {
    uint32_t lo = off[b], hi = off[b + 1];
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t v = keys[mid];
        if (v == a) return true;
        if (v < a) lo = mid + 1;
        else hi = mid;
    }
    return false;
}
// current pair (a, b), or -1 (the B-side list of b is in ascending a)
static __device__ __forceinline__ int32_t find_pair(const DW& w, uint32_t a, uint32_t b) {
    uint32_t lo = w.offB[b], hi = w.offB[b + 1];
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t p = w.listB[mid];
        uint32_t v = w.p_ab[p].x;
        if (v == a) return (int32_t)p;
        if (v < a) lo = mid + 1;
        else hi = mid;
    }
    return -1;
}

struct TouchSets {
    const uint32_t *poff, *pkeys;  // previous set
    const uint32_t* noff;          // next set: its offsets (the scanned touch counts) ...
    uint32_t* nkeys;               // ... and keys
};
static __device__ __forceinline__ TouchSets touch_sets(const DW& w) {
    uint32_t par = w.evs[EV_PAR] & 1u;
    TouchSets t;
    t.poff = w.toff;
    t.pkeys = par ? w.tk1 : w.tk0;
    t.noff = w.ev_ct;
    t.nkeys = par ? w.tk0 : w.tk1;
    return t;
}

// Merge of body b's touching pairs (ascending a) with its previous list
// (ascending a).  Visit(kind, a, p): kind 0 begin, 1 end, 3 still touching.
template <class F>
static __device__ __forceinline__ void merge_touch(const DW& w, const TouchSets& t, uint32_t b, F visit) {
    uint32_t i = w.offB[b], i1 = w.offB[b + 1];
    uint32_t j = t.poff[b], j1 = t.poff[b + 1];
    for (;;) {
        while (i < i1 && !(w.t_flag[w.listB[i]] & 1u)) i++;
        bool hi = i < i1, hj = j < j1;
        if (!hi && !hj) break;
        uint32_t p = hi ? w.listB[i] : 0u;
        uint32_t a_cur = hi ? w.p_ab[p].x : 0xffffffffu;
        uint32_t a_prev = hj ? t.pkeys[j] : 0xffffffffu;
        if (hi && (!hj || a_cur < a_prev)) {
            visit(0, a_cur, p);
            i++;
        } else if (hj && (!hi || a_prev < a_cur)) {
            visit(1, a_prev, 0u);
            j++;
        } else {
            visit(3, a_cur, p);
            i++;
            j++;
        }
    }
}

// Swept-hit event of mover h, unless this substep reports a hit for the pair.
static __device__ __forceinline__ bool ccd_event_kept(const DW& w, const TouchSets& t, uint32_t h, int emit) {
    int32_t o = w.ccd_ev_o[h];
    if (o < 0) return false;
    if (!emit) return true;
    uint32_t lo = min(h, (uint32_t)o), hi = max(h, (uint32_t)o);
    int32_t p = find_pair(w, lo, hi);
    if (p < 0 || !(w.t_flag[p] & 1u)) return true;
    bool began = !in_touch_set(t.poff, t.pkeys, lo, hi);
    return !(began && w.t_wit[p].w > CONTACT_HIT_THRESHOLD);
}

// pass 1: per-body counts (cnt arrays hold N+1 entries, the last one 0)
__global__ void k_ev_count(DW w, int emit) {
    if (aborted_solve(w)) return;
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > (uint32_t)w.N) return;
    if (b == (uint32_t)w.N) {
        w.ev_cbe[b] = 0;
        w.ev_ch[b] = 0;
        w.ev_cc[b] = 0;
        w.ev_ct[b] = 0;
        return;
    }
    TouchSets t = touch_sets(w);
    uint32_t nbe = 0, nh = 0, nt = 0;
    if (emit) {
        merge_touch(w, t, b, [&](int kind, uint32_t, uint32_t p) {
            if (kind != 1) nt++;
            if (kind == 1 || kind == 0) nbe++;
            if (kind == 0 && w.t_wit[p].w > CONTACT_HIT_THRESHOLD) nh++;
        });
    }
    w.ev_ct[b] = nt;
    w.ev_cbe[b] = nbe;
    w.ev_ch[b] = nh;
    w.ev_cc[b] = (w.ccd_ev_o && ccd_event_kept(w, t, b, emit)) ? 1u : 0u;
}

static __device__ __forceinline__ void put_event(const DW& w, uint32_t pos, uint32_t a, uint32_t b, uint32_t kind,
                                                 V3 pt, V3 nrm, float approach) {
    if (pos >= w.ev_cap) return;
    AvbdContactEvent e;
    e.body_a = a;
    e.body_b = b;
    e.kind = kind;
    e.point[0] = pt.x;
    e.point[1] = pt.y;
    e.point[2] = pt.z;
    e.normal[0] = nrm.x;
    e.normal[1] = nrm.y;
    e.normal[2] = nrm.z;
    e.approach_speed = approach;
    w.ev[pos] = e;
}

// pass 2: write the events at their scanned slots and the next touch set
__global__ void k_ev_write(DW w, int emit) {
    if (aborted_solve(w)) return;
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= (uint32_t)w.N) return;
    const uint32_t N = (uint32_t)w.N;
    const uint32_t base = w.evs[EV_N];
    const uint32_t tot_be = emit ? w.ev_cbe[N] : 0u, tot_h = emit ? w.ev_ch[N] : 0u;
    TouchSets t = touch_sets(w);
    if (emit) {
        uint32_t pbe = base + w.ev_cbe[b], ph = base + tot_be + w.ev_ch[b], pt = t.noff[b];
        merge_touch(w, t, b, [&](int kind, uint32_t a, uint32_t p) {
            if (kind != 1) t.nkeys[pt++] = a;
            if (kind == 0) {
                put_event(w, pbe++, a, b, AVBD_CONTACT_BEGIN, V0(), V0(), 0.0f);
                float4 wt = w.t_wit[p];
                if (wt.w > CONTACT_HIT_THRESHOLD)
                    put_event(w, ph++, a, b, AVBD_CONTACT_HIT, ld3(wt), -ld3(w.p_n[p]), wt.w);
            } else if (kind == 1) {
                put_event(w, pbe++, a, b, AVBD_CONTACT_END, V0(), V0(), 0.0f);
            }
        });
    }
    if (w.ccd_ev_o && ccd_event_kept(w, t, b, emit)) {
        uint32_t o = (uint32_t)w.ccd_ev_o[b];
        float4 pp = w.ccd_ev_p[b];
        put_event(w, base + tot_be + tot_h + w.ev_cc[b], min(b, o), max(b, o), AVBD_CONTACT_HIT, ld3(pp),
                  ld3(w.ccd_ev_n[b]), pp.w);
    }
}

// the next touch set replaces the previous one: its offsets move into toff
__global__ void k_ev_commit(DW w) {
    if (aborted_solve(w)) return;
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b <= (uint32_t)w.N) w.toff[b] = w.ev_ct[b];
}
__global__ void k_ev_finish(DW w, int emit) {
    if (aborted_solve(w) || threadIdx.x != 0) return;
    const uint32_t N = (uint32_t)w.N;
    uint32_t total = w.ev_cc[N] + (emit ? w.ev_cbe[N] + w.ev_ch[N] : 0u);
    uint32_t n = w.evs[EV_N] + total;
    if (n > w.ev_cap) {
        w.evs[EV_DROP] += n - w.ev_cap;
        n = w.ev_cap;
    }
    w.evs[EV_N] = n;
    if (emit) w.evs[EV_PAR] ^= 1u;
}

// ---- triggers ------------------------------------------------------------------
constexpr int TRIG_SORT_THREADS = 512;
// One CTA: sort this substep's overlaps by (b, a), diff them against the
// previous set (same order), queue Entered / Exited, keep the new set.
__global__ void __launch_bounds__(TRIG_SORT_THREADS) k_trig_events(DW w) {
    if (aborted_solve(w)) return;
    __shared__ unsigned long long key[TRIG_CAP];
    uint32_t n = min(w.evs[EV_TRIG_NOW], (uint32_t)TRIG_CAP);
    uint32_t m = 1;
    while (m < n) m <<= 1;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) key[i] = i < n ? w.trig_now[i] : ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= m; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
                uint32_t l = i ^ j;
                if (l > i) {
                    unsigned long long x = key[i], y = key[l];
                    bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        key[i] = y;
                        key[l] = x;
                    }
                }
            }
            __syncthreads();
        }
    if (threadIdx.x == 0) {
        uint32_t np = w.evs[EV_TRIG_PREV], i = 0, j = 0, q = w.evs[EV_TN];
        auto put = [&](unsigned long long k, uint32_t entered) {
            if (q < w.tev_cap) w.tev[q] = AvbdTriggerEvent{(uint32_t)(k & 0xffffffffu), (uint32_t)(k >> 32), entered};
            else w.evs[EV_TDROP]++;
            q++;
        };
        while (i < n || j < np) {
            unsigned long long x = i < n ? key[i] : ~0ull, y = j < np ? w.trig_prev[j] : ~0ull;
            if (x < y) { put(x, 1u); i++; }
            else if (y < x) { put(y, 0u); j++; }
            else { i++; j++; }
        }
        w.evs[EV_TN] = min(q, w.tev_cap);
        w.evs[EV_TRIG_PREV] = n;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) w.trig_prev[i] = key[i];
}

void launch_events(const DW& w, int emit, int triggers, uint32_t* scan_tmp, cudaStream_t st) {
    if (!w.evs) return;
    unsigned g1 = nblk((size_t)w.N + 1, 256), gb = nblk(w.N, 256);
    if (emit) k_ev_touch<<<gsz(w.pair_cap, 256), 256, 0, st>>>(w);
    k_ev_count<<<g1, 256, 0, st>>>(w, emit);
    scan_exclusive(w.ev_cbe, w.ev_cbe, (size_t)w.N + 1, scan_tmp, st);
    scan_exclusive(w.ev_ch, w.ev_ch, (size_t)w.N + 1, scan_tmp, st);
    scan_exclusive(w.ev_cc, w.ev_cc, (size_t)w.N + 1, scan_tmp, st);
    if (emit) scan_exclusive(w.ev_ct, w.ev_ct, (size_t)w.N + 1, scan_tmp, st);
    k_ev_write<<<gb, 256, 0, st>>>(w, emit);
    if (emit) k_ev_commit<<<g1, 256, 0, st>>>(w);
    k_ev_finish<<<1, 32, 0, st>>>(w, emit);
    if (emit && triggers) k_trig_events<<<1, TRIG_SORT_THREADS, 0, st>>>(w);
}

}  // namespace avbd
