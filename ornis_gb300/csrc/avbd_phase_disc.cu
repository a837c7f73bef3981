// avbd_phase_disc.cu — pair discovery (narrowphase, manifold, warm merge),
// the per-body incidence lists, inertial targets, warmstart decay and the
// body colouring.
//
// Reference: crates/physics/src/avbd/rows.rs:303-343 (contact normal frame),
// :432-756 (discover_pair), :767-943 (generate_pairs merge),
// avbd/mod.rs:980-1049 (wake, targets, decay).
#include "avbd_common.cuh"

namespace avbd {

void launch_wake_apply(const DW& w, cudaStream_t st);

struct Disc {
    bool keep, exists, separated;
    int32_t old;  // index of the previous-generation pair, -1 when new
    V3 normal;
    float sgn, ra, rb;
    Dist d;
};

// discover_pair (rows.rs:432-555) in three parts: the prefilter and the
// previous-generation lookup; the signed gap with witnesses; the contact
// frame and the creation gate.
static __device__ __forceinline__ bool discover_pre(const DW& w, uint32_t a, uint32_t b, Disc& r) {
    r.keep = false;
    r.exists = false;
    r.separated = false;
    r.old = -1;
    if (!pair_allowed(w, a, b)) return false;
    if (info_trigger(w.info[a]) || info_trigger(w.info[b])) return false;  // triggers form no contact pair here
    if (jointed_no_collide(w, a, b)) return false;
    r.ra = w.shp[a].w;
    r.rb = w.shp[b].w;
    if (len(ld3(w.pos[a]) - ld3(w.pos[b])) > r.ra + r.rb + GEN_MARGIN) return false;
    r.old = find_old_pair(w, a, b);
    r.exists = r.old >= 0;
    return true;
}
static __device__ __forceinline__ void discover_post(const DW& w, uint32_t a, uint32_t b, const Shape& sa,
                                                     const Shape& sb, Disc& r) {
    V3 normal;
    if (sa.kind == AVBD_SHAPE_HALFSPACE) normal = -qrot(sa.rot, sa.p);
    else if (sb.kind == AVBD_SHAPE_HALFSPACE) normal = qrot(sb.rot, sb.p);
    else {
        V3 nm = r.d.pa - r.d.pb;
        if (r.d.dist < 0.0f) nm = -nm;
        if (len2(nm) < AXIS_REST_LEN2) nm = sa.pos - sb.pos;
        nm = normalize_or(nm, VY());
        if (r.exists) {
            if (dot(nm, ld3(w.o_n[r.old])) < 0.0f) nm = -nm;
        } else if (dot(nm, sa.pos - sb.pos) < 0.0f) {
            nm = -nm;
        }
        normal = nm;
    }
    r.normal = normal;
    float approach = fmaxf(dot(ld3(w.vel[b]) - ld3(w.vel[a]), normal), 0.0f);
    float reach = GEN_MARGIN + approach * w.dt;
    if (r.sgn > reach && !r.exists) return;
    r.separated = r.sgn > reach;
    r.keep = true;
}
static __device__ __noinline__ Disc discover(const DW& w, uint32_t a, uint32_t b, bool need_witness) {
    Disc r;
    if (!discover_pre(w, a, b, r)) return r;
    if (r.exists && !need_witness) {
        // live pairs within the prefilter always survive (empty shells are
        // kept, rows.rs:555-564): the filter pass needs no distance for them
        r.keep = true;
        return r;
    }
    Shape sa = shape_of(w, a), sb = shape_of(w, b);
    bool boxes = sa.kind == AVBD_SHAPE_BOX && sb.kind == AVBD_SHAPE_BOX;
    if (boxes && !r.exists && !need_witness) {
        // The signed gap of a box pair is the SAT gap (rows.rs:498-510) and the
        // creation reach is at most GEN_MARGIN + |v_b - v_a| dt: a new pair
        // beyond that is rejected without the witness features.
        V3 nsat;
        float gap = separating_axis(sa.pos, sa.rot, sa.p, sb.pos, sb.rot, sb.p, nsat);
        float bound = GEN_MARGIN + len(ld3(w.vel[b]) - ld3(w.vel[a])) * w.dt * 1.00001f + 1e-6f;
        if (gap > bound) return r;
    }
    float sat = 0.0f;
    r.d = ext_distance(w, sa, sb, &sat);
    r.sgn = boxes ? sat : r.d.dist;
    discover_post(w, a, b, sa, sb, r);
    return r;
}

// A trigger pair overlaps when discover_pair would report it with a signed
// gap <= 0 (rows.rs:432-520: no joint exclusion for triggers).
static __device__ __noinline__ bool trigger_overlap(const DW& w, uint32_t a, uint32_t b) {
    if (!pair_allowed(w, a, b)) return false;
    if (len(ld3(w.pos[a]) - ld3(w.pos[b])) > w.shp[a].w + w.shp[b].w + GEN_MARGIN) return false;
    Shape sa = shape_of(w, a), sb = shape_of(w, b);
    float sat = 0.0f;
    Dist d = ext_distance(w, sa, sb, &sat);
    float sgn = (sa.kind == AVBD_SHAPE_BOX && sb.kind == AVBD_SHAPE_BOX) ? sat : d.dist;
    return sgn <= 0.0f;
}
static __device__ __forceinline__ void k_disc_filter_one(const DW& w, uint32_t c, int triggers) {
    uint2 ab = w.cand[c];
    if (triggers && (info_trigger(w.info[ab.x]) || info_trigger(w.info[ab.y]))) {
        w.keep[c] = 0;
        if (trigger_overlap(w, ab.x, ab.y)) {
            uint32_t slot = agg_inc(&w.evs[EV_TRIG_NOW]);
            if (slot < (uint32_t)TRIG_CAP) w.trig_now[slot] = ((unsigned long long)ab.y << 32) | ab.x;
            else w.evs[EV_TRIG_OVF] = 1u;
        }
        return;
    }
    Disc d = discover(w, ab.x, ab.y, false);
    w.keep[c] = d.keep;
    if (d.keep) agg_inc_at(w.cnt, ab.x);
}
__global__ void __launch_bounds__(128, 4) k_disc_filter(DW w, int triggers) {
    if (aborted(w)) return;
    const uint32_t n = n_cand(w);
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        k_disc_filter_one(w, c, triggers);
}

static __device__ __forceinline__ void k_place_one(const DW& w, uint32_t c) {
    if (!w.keep[c]) return;
    uint32_t a = w.cand[c].x;
    w.slot_c[w.offA[a] + agg_inc_at(w.cur, a)] = c;
}
__global__ void k_place(DW w) {
    if (aborted(w)) return;
    const uint32_t n = n_cand(w);
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        k_place_one(w, c);
}

// Each dynamic body's A-side slots in ascending b, so a swept body visits its
// pairs in the reference's order.  The segments of static bodies
// (half-spaces, floors: often long) are never read in sequence and are left
// as placed, unless the world keeps a differentiable rollout: its adjoint
// carries point state across checkpoints by pair index, so every segment is
// put in one order.  A thread sorts a short segment by insertion; a long
// static one (a floor under thousands of bodies) is listed for the chunk
// sort below.
constexpr uint32_t SORT_SHORT = 64;
constexpr uint32_t SORT_CHUNK = 1024;
__global__ void k_sort_slots(DW w) {
    if (aborted(w)) return;
    uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= (uint32_t)w.N) return;
    if (a == 0) w.ctr[C_PAIRS] = w.offA[w.N];
    uint32_t s0 = w.offA[a], s1 = w.offA[a + 1];
    if (!is_dynamic(w, a)) {
        if (!w.sort_static) return;
        if (s1 - s0 > SORT_SHORT) {
            w.long_seg[atomicAdd(&w.ctr[C_LONGSEG], 1u)] = a;
            return;
        }
    }
    for (uint32_t i = s0 + 1; i < s1; i++) {
        uint32_t c = w.slot_c[i];
        uint32_t bk = w.cand[c].y;
        uint32_t k = i;
        while (k > s0 && w.cand[w.slot_c[k - 1]].y > bk) {
            w.slot_c[k] = w.slot_c[k - 1];
            k--;
        }
        w.slot_c[k] = c;
    }
}

// Manifold (rows.rs:571-715), wake vote (:716-744) and warm merge with the
// previous generation (:809-931) for one surviving pair.
static __device__ __forceinline__ bool box_pair(const DW& w, uint2 ab) {
    return info_shape(w.info[ab.x]) == AVBD_SHAPE_BOX && info_shape(w.info[ab.y]) == AVBD_SHAPE_BOX;
}
// Box-box witnesses are computed ahead, one thread per box pair, into bd_pa /
// bd_pb; the per-pair build below then reads them.  Every box pair runs the
// same fixed loops (15 SAT axes, 16 corner and 144 edge tests), so a warp of
// box pairs stays converged and the kernel is ALU-bound with few loads.
// Pairs are built class by class (box-box, one box, no box) so the lanes of
// a warp run the same manifold code: corners of two boxes, of one, or none.
static __device__ __forceinline__ void k_collect_boxes_one(const DW& w, uint32_t p) {
    uint2 ab = w.cand[w.slot_c[p]];
    int boxes = (info_shape(w.info[ab.x]) == AVBD_SHAPE_BOX) + (info_shape(w.info[ab.y]) == AVBD_SHAPE_BOX);
    if (boxes == 2) w.boxlist[agg_inc(&w.ctr[C_BOXPAIRS])] = p;
    else if (boxes == 1) w.boxlist[w.pair_cap - 1u - agg_inc(&w.ctr[C_BOXONE])] = p;
    else w.clist[agg_inc(&w.ctr[C_NOBOX])] = p;
}
__global__ void k_collect_boxes(DW w) {
    if (aborted(w)) return;
    const uint32_t n = n_pairs(w);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        k_collect_boxes_one(w, p);
}
__global__ void k_box_witness(DW w) {
    if (aborted(w)) return;
    const uint32_t nbox = w.ctr[C_BOXPAIRS];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nbox; i += gridDim.x * blockDim.x) {
        uint32_t p = w.boxlist[i];
        uint2 ab = w.cand[w.slot_c[p]];
        Shape sa = shape_of(w, ab.x), sb = shape_of(w, ab.y);
        float sat;
        Dist d = box_box(sa.pos, sa.rot, sa.p, sb.pos, sb.rot, sb.p, &sat);
        w.bd_pa[p] = st3(d.pa, d.dist);
        w.bd_pb[p] = st3(d.pb, sat);
    }
}
static __device__ __forceinline__ void build_pair(const DW& w, uint32_t p, uint2 ab, const Disc& d);
static __device__ __forceinline__ void k_disc_build_one(const DW& w, uint32_t p) {
    uint32_t c = w.slot_c[p];
    uint2 ab = w.cand[c];
    if (box_pair(w, ab)) {
        Disc r;
        discover_pre(w, ab.x, ab.y, r);  // passed in the filter pass: same state, same result
        float4 pa = w.bd_pa[p], pb = w.bd_pb[p];
        r.d = Dist{pa.w, ld3(pa), ld3(pb)};
        r.sgn = pb.w;
        discover_post(w, ab.x, ab.y, shape_of(w, ab.x), shape_of(w, ab.y), r);
        build_pair(w, p, ab, r);
        return;
    }
    build_pair(w, p, ab, discover(w, ab.x, ab.y, true));
}
static __device__ __forceinline__ void build_pair(const DW& w, uint32_t p, uint2 ab, const Disc& d) {
    uint32_t ia = ab.x, ib = ab.y;
    V3 normal = d.normal;
    float sgn = d.sgn;
    float mu = fmaxf(fmaxf(w.mat[ia].y, w.mat[ib].y), 0.0f);
    V3 posa = ld3(w.pos[ia]), posb = ld3(w.pos[ib]);
    Q qa = ldq(w.rot[ia]), qb = ldq(w.rot[ib]);
    uint32_t ka = info_shape(w.info[ia]), kb = info_shape(w.info[ib]);
    float4 spa = w.shp[ia], spb = w.shp[ib];
    V3 fra[MAX_PTS], frb[MAX_PTS];
    int nf = 0;
    float patch = fminf(d.ra, d.rb) + MARGIN;
    V3 pp = (d.d.pa + d.d.pb) * HALF;
    V3 pa_c = posa - normal * dot(posa - pp, normal);
    V3 pb_c = posb - normal * dot(posb - pp, normal);
    float plane_a = ka == AVBD_SHAPE_BOX ? dot(normal, posa) - 1.0f * dot(vabs(qrot(conj(qa), normal)), ld3(spa))
                                         : dot(normal, d.d.pa);
    float plane_b = kb == AVBD_SHAPE_BOX
                        ? dot(normal, posb) - (-1.0f) * dot(vabs(qrot(conj(qb), normal)), ld3(spb))
                        : dot(normal, d.d.pb);
    Q inv_a = conj(qa), inv_b = conj(qb);
    auto dup = [&](V3 ral, V3 rbl) {
        for (int k = 0; k < nf; k++)
            if (len(fra[k] - ral) < POINT_MATCH_DIST && len(frb[k] - rbl) < POINT_MATCH_DIST) return true;
        return false;
    };
    if (!d.separated) {
        for (int side = 0; side < 2; side++) {
            if ((side == 0 ? ka : kb) != AVBD_SHAPE_BOX) continue;
            V3 bpos = side == 0 ? posa : posb;
            Q brot = side == 0 ? qa : qb;
            V3 half = ld3(side == 0 ? spa : spb);
            V3 witness = side == 0 ? d.d.pa : d.d.pb;
            float sign = side == 0 ? 1.0f : -1.0f;
            V3 pc = side == 0 ? pa_c : pb_c;
            for (int ci = 0; ci < 8; ci++) {
                // corner order of rows.rs:346-363: x outer, z inner, - before +
                float sx = (ci & 4) ? 1.0f : -1.0f, sy = (ci & 2) ? 1.0f : -1.0f, sz = (ci & 1) ? 1.0f : -1.0f;
                V3 corner{sx * half.x, sy * half.y, sz * half.z};
                V3 world = bpos + qrot(brot, corner);
                float along = dot(world - witness, sign * normal);
                if (fabsf(along) > EXPAND_SLOP + fmaxf(-sgn, 0.0f)) continue;
                V3 rel = world - pc;
                V3 tang = rel - normal * dot(rel, normal);
                if (len(tang) > patch) continue;
                if (nf >= MAX_PTS) break;
                V3 pa, pb;
                if (side == 0) {
                    pa = world;
                    pb = world + normal * (plane_b - dot(normal, world));
                } else {
                    pa = world + normal * (plane_a - dot(normal, world));
                    pb = world;
                }
                V3 ral = qrot(inv_a, pa - posa), rbl = qrot(inv_b, pb - posb);
                if (dup(ral, rbl)) continue;
                fra[nf] = ral;
                frb[nf] = rbl;
                nf++;
            }
        }
    }
    if (!d.separated && nf >= 2 && nf < MAX_PTS) {
        V3 mid = d.ra < d.rb ? pa_c : (d.rb < d.ra ? pb_c : (pa_c + pb_c) * HALF);
        V3 pa = mid + normal * (plane_a - dot(normal, mid));
        V3 pb = mid + normal * (plane_b - dot(normal, mid));
        V3 ral = qrot(inv_a, pa - posa), rbl = qrot(inv_b, pb - posb);
        if (!dup(ral, rbl)) {
            fra[nf] = ral;
            frb[nf] = rbl;
            nf++;
        }
    }
    if (!d.separated && nf < 3) {
        V3 ral = qrot(inv_a, d.d.pa - posa), rbl = qrot(inv_b, d.d.pb - posb);
        if (!dup(ral, rbl)) {
            fra[nf] = ral;
            frb[nf] = rbl;
            nf++;
        }
    }
    bool wake;
    if (d.exists) {
        wake = (w.asleep[ia] || w.asleep[ib]) && sgn < -WAKE_PENETRATION;
    } else {
        bool impact = sgn < -WAKE_PENETRATION;
        if (!impact && w.asleep[ia]) impact = dot(ld3(w.vel[ib]) - ld3(w.vel[ia]), 1.0f * normal) > WAKE_IMPACT_SPEED;
        if (!impact && w.asleep[ib])
            impact = dot(ld3(w.vel[ia]) - ld3(w.vel[ib]), -1.0f * normal) > WAKE_IMPACT_SPEED;
        wake = impact;
    }
    if (wake) {
        w.flag[ia] = 1;
        w.flag[ib] = 1;
    }
    w.p_ab[p] = ab;
    w.p_n[p] = st3(normal, sgn);
    w.p_mu[p] = make_float2(mu, mu);
    w.p_np[p] = (uint32_t)nf;
    if (w.p_old) w.p_old[p] = d.exists ? d.old : -1;
    bool touching = sgn <= 0.0f;
    bool smooth = ka == AVBD_SHAPE_SPHERE || kb == AVBD_SHAPE_SPHERE;
    uint32_t onp = d.exists ? w.o_np[d.old] : 0u;
    for (int k = 0; k < nf; k++) {
        uint32_t q = p * MAX_PTS + k;
        int m = -1;
        for (uint32_t j = 0; j < onp; j++) {
            float4 ora = w.oq_ra[(uint32_t)d.old * MAX_PTS + j];
            if (len(ld3(ora) - fra[k]) < LAMBDA_MATCH_DIST) {
                m = (int)j;
                break;
            }
        }
        if (m >= 0) {
            uint32_t oq = (uint32_t)d.old * MAX_PTS + m;
            float4 ora = w.oq_ra[oq], orb = w.oq_rb[oq];
            if (orb.w != 0.0f && touching && !smooth) {  // stuck: anchors stay frozen (q_ra.w = 1: kept)
                w.q_ra[q] = make_float4(ora.x, ora.y, ora.z, 1.0f);
                w.q_rb[q] = orb;
            } else {
                w.q_ra[q] = st3(fra[k], 0.0f);
                w.q_rb[q] = st3(frb[k], orb.w);
            }
            w.q_lam[q] = w.oq_lam[oq];
            w.q_pen[q] = w.oq_pen[oq];
            w.q_roll[q] = w.oq_roll[oq];
        } else {
            w.q_ra[q] = st3(fra[k], 0.0f);
            w.q_rb[q] = st3(frb[k], 1.0f);
            w.q_lam[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w.q_pen[q] = make_float4(PENALTY_INIT, PENALTY_INIT, PENALTY_INIT, 0.0f);
            w.q_roll[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        w.q_matched[q] = m;
    }
    agg_add(&w.ctr[C_POINTS], (uint32_t)nf);
}
// cls 0: box-box pairs, 1: one box, 2: no box
__global__ void __launch_bounds__(128, 4) k_disc_build(DW w, int cls) {
    if (aborted(w)) return;
    const uint32_t n = w.ctr[cls == 0 ? C_BOXPAIRS : (cls == 1 ? C_BOXONE : C_NOBOX)];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t p = cls == 0 ? w.boxlist[i] : (cls == 1 ? w.boxlist[w.pair_cap - 1u - i] : w.clist[i]);
        k_disc_build_one(w, p);
    }
}

__global__ void k_clear_flags(DW w) {
    if (aborted(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < (uint32_t)w.N) w.flag[h] = 0;
}

// Long static segments, in (b, candidate) order: every chunk of SORT_CHUNK
// slots is sorted in shared memory (bitonic network), then each slot's final
// place is its place in its chunk plus, for every other chunk, the number of
// smaller keys there (binary search).  Keys are unique (one candidate per
// slot), so the places are a permutation of the segment.
__global__ void __launch_bounds__(512) k_sort_long_chunks(DW w) {
    if (aborted(w)) return;
    const uint32_t nl = w.ctr[C_LONGSEG];
    __shared__ unsigned long long key[SORT_CHUNK];
    for (uint32_t l = 0; l < nl; l++) {
        const uint32_t a = w.long_seg[l];
        const uint32_t s0 = w.offA[a], s1 = w.offA[a + 1];
        const uint32_t nch = (s1 - s0 + SORT_CHUNK - 1) / SORT_CHUNK;
        for (uint32_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
            const uint32_t c0 = s0 + ch * SORT_CHUNK, len = min(SORT_CHUNK, s1 - c0);
            for (uint32_t i = threadIdx.x; i < SORT_CHUNK; i += blockDim.x) {
                unsigned long long k = ~0ull;
                if (i < len) {
                    uint32_t c = w.slot_c[c0 + i];
                    k = ((unsigned long long)w.cand[c].y << 32) | c;
                }
                key[i] = k;
            }
            __syncthreads();
            for (uint32_t k = 2; k <= SORT_CHUNK; k <<= 1)
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t t = threadIdx.x; t < SORT_CHUNK / 2; t += blockDim.x) {
                        uint32_t i = 2 * t - (t & (j - 1));  // t with a zero bit inserted at j
                        unsigned long long x = key[i], y = key[i + j];
                        if ((x > y) == ((i & k) == 0)) {
                            key[i] = y;
                            key[i + j] = x;
                        }
                    }
                    __syncthreads();
                }
            for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) w.seg_key[c0 + i] = key[i];
            __syncthreads();
        }
    }
}
__global__ void k_sort_long_rank(DW w) {
    if (aborted(w)) return;
    const uint32_t nl = w.ctr[C_LONGSEG];
    for (uint32_t l = 0; l < nl; l++) {
        const uint32_t a = w.long_seg[l];
        const uint32_t s0 = w.offA[a], n = w.offA[a + 1] - s0;
        const unsigned long long* sk = w.seg_key + s0;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const unsigned long long k = sk[i];
            const uint32_t own = i / SORT_CHUNK;
            uint32_t place = i - own * SORT_CHUNK;
            for (uint32_t lo = 0, ch = 0; lo < n; lo += SORT_CHUNK, ch++) {
                if (ch == own) continue;
                uint32_t b0 = lo, b1 = min(lo + SORT_CHUNK, n);
                while (b0 < b1) {
                    uint32_t m = (b0 + b1) >> 1;
                    if (sk[m] < k) b0 = m + 1;
                    else b1 = m;
                }
                place += b0 - lo;
            }
            w.slot_c[s0 + place] = (uint32_t)(k & 0xffffffffull);
        }
    }
}

void launch_discovery(const DW& w, uint32_t* scan_tmp, cudaStream_t st, int triggers) {
    unsigned g1 = nblk(w.N + 1, 256);
    k_zero_u32<<<g1, 256, 0, st>>>(w.cnt, w.N + 1);
    k_zero_u32<<<g1, 256, 0, st>>>(w.cur, w.N + 1);
    k_disc_filter<<<gsz(w.cand_cap, 128), 128, 0, st>>>(w, triggers && w.evs ? 1 : 0);
    scan_exclusive(w.cnt, w.offA, w.N + 1, scan_tmp, st);
    k_place<<<gsz(w.cand_cap, 256), 256, 0, st>>>(w);
    k_sort_slots<<<nblk(w.N, 256), 256, 0, st>>>(w);
    if (w.sort_static) {
        k_sort_long_chunks<<<2 * 152, 512, 0, st>>>(w);
        k_sort_long_rank<<<4 * 152, 256, 0, st>>>(w);
    }
    k_clear_flags<<<nblk(w.N, 256), 256, 0, st>>>(w);
    k_collect_boxes<<<gsz(w.pair_cap, 256), 256, 0, st>>>(w);
    k_box_witness<<<gsz(w.pair_cap, 128), 128, 0, st>>>(w);
    for (int cls = 0; cls < 3; cls++) k_disc_build<<<gsz(w.pair_cap, 128), 128, 0, st>>>(w, cls);
}

// ---- after discovery ----------------------------------------------------------
// mod.rs:985-992: a sleeper kicked above the thresholds wakes before warmstart
__global__ void k_external_wake(DW w) {
    if (aborted(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N || !w.asleep[h]) return;
    if (len(ld3(w.vel[h])) > SLEEP_LIN || len(ld3(w.angvel[h])) > SLEEP_ANG) wake_body(w, h);
}
static __device__ __forceinline__ void k_countB_one(const DW& w, uint32_t p) {
    atomicAdd(&w.cnt[w.p_ab[p].y], 1u);
}
__global__ void k_countB(DW w) {
    if (aborted(w)) return;
    const uint32_t n = n_pairs(w);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        k_countB_one(w, p);
}

static __device__ __forceinline__ void k_placeB_one(const DW& w, uint32_t p) {
    uint32_t b = w.p_ab[p].y;
    w.listB[w.offB[b] + atomicAdd(&w.cur[b], 1u)] = p;
}
__global__ void k_placeB(DW w) {
    if (aborted(w)) return;
    const uint32_t n = n_pairs(w);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        k_placeB_one(w, p);
}

__global__ void k_sortB(DW w) {
    if (aborted(w)) return;
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= (uint32_t)w.N) return;
    uint32_t s0 = w.offB[b], s1 = w.offB[b + 1];
    for (uint32_t i = s0 + 1; i < s1; i++) {
        uint32_t v = w.listB[i];
        uint32_t k = i;
        while (k > s0 && w.listB[k - 1] > v) {
            w.listB[k] = w.listB[k - 1];
            k--;
        }
        w.listB[k] = v;
    }
    if (w.posB)
        for (uint32_t i = s0; i < s1; i++) w.posB[w.listB[i]] = i;
}
// mod.rs:993-1018 (step-start pose, inertial target) and :1043-1049 (x <- y)
__global__ void k_targets(DW w) {
    if (aborted(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    float4 p = w.pos[h], q = w.rot[h];
    if (info_type(w.info[h]) == AVBD_BODY_KINEMATIC) {
        w.pos0[h] = w.prev_pos[h];
        w.rot0[h] = w.prev_rot[h];
    } else {
        w.pos0[h] = p;
        w.rot0[h] = q;
    }
    if (!solvable(w, h)) {
        w.inertial[h] = p;
        w.inertial_rot[h] = q;
        return;
    }
    float dt = w.dt;
    V3 y = ld3(p) + ld3(w.vel[h]) * dt + w.gravity * (dt * dt);
    Q qt = quat_integrate(ldq(q), ld3(w.angvel[h]) * dt);
    w.inertial[h] = st3(y, 0.0f);
    w.inertial_rot[h] = stq(qt);
    if (!w.asleep[h]) {
        w.pos[h] = st3(y, 0.0f);
        w.rot[h] = stq(qt);
    }
}
// Contact record of every body for the iterations (pose, x - x0,
// quat_diff_vec(q, q0), shape word and first parameter in one 64-byte line),
// taken at the start of the sweep; the primal refreshes a body's record when
// it moves it.
__global__ void k_motion_cache(DW w) {
    if (aborted(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    V3 p = ld3(w.pos[h]);
    Q q = ldq(w.rot[h]);
    V3 dx = p - ld3(w.pos0[h]);
    V3 dr = quat_diff_vec(q, ldq(w.rot0[h]));
    float4* k = w.kin + (size_t)h * 4;
    k[0] = st3(p, w.shp[h].x);
    k[1] = stq(q);
    k[2] = st3(dx, __uint_as_float(w.info[h]));
    k[3] = st3(dr, 0.0f);
}
// Eq. 19 warmstart decay (mod.rs:1019-1040), then the point's step-start
// normal violation C0 (joints_ext.rs:21-32), kept in lambda.w for the
// iterations of this substep.
static __device__ __forceinline__ void k_decay_points_one(const DW& w, uint32_t q) {
    uint32_t p = q / MAX_PTS, k = q % MAX_PTS;
    if (k >= w.p_np[p]) return;
    const float ag = ALPHA * GAMMA;
    float4 l = w.q_lam[q], r = w.q_roll[q], pn = w.q_pen[q];
    float4 n4 = w.p_n[p];
    float c0 = 0.0f;
    if (n4.w <= 0.0f) {
        uint2 ab = w.p_ab[p];
        bool sph = info_shape(w.info[ab.x]) == AVBD_SHAPE_SPHERE || info_shape(w.info[ab.y]) == AVBD_SHAPE_SPHERE;
        c0 = gap_c0(sph, n4.w, ld3(n4), ld3(w.pos0[ab.x]), ldq(w.rot0[ab.x]), ld3(w.pos0[ab.y]), ldq(w.rot0[ab.y]),
                    w.q_ra[q], w.q_rb[q]);
    }
    w.q_lam[q] = make_float4(l.x * ag, l.y * ag, l.z * ag, c0);
    w.q_roll[q] = make_float4(r.x * ag, r.y * ag, r.z * ag, 0.0f);
    w.q_pen[q] = make_float4(fclamp(pn.x * GAMMA, PENALTY_MIN, PENALTY_MAX),
                             fclamp(pn.y * GAMMA, PENALTY_MIN, PENALTY_MAX),
                             fclamp(pn.z * GAMMA, PENALTY_MIN, PENALTY_MAX), 0.0f);
}
__global__ void k_decay_points(DW w) {
    if (aborted(w)) return;
    const uint32_t n = n_pairs(w) * MAX_PTS;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
        k_decay_points_one(w, q);
}
__global__ void k_decay_joints(DW w) {
    if (aborted(w)) return;
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (uint32_t)w.J) return;
    const float ag = ALPHA * GAMMA;
    float4 a = w.j_lam_l[j], b = w.j_lam_a[j], c = w.j_pen_l[j], d = w.j_pen_a[j];
    w.j_lam_l[j] = make_float4(a.x * ag, a.y * ag, a.z * ag, 0.0f);
    w.j_lam_a[j] = make_float4(b.x * ag, b.y * ag, b.z * ag, 0.0f);
    float4 pl = make_float4(fclamp(c.x * GAMMA, PENALTY_MIN, PENALTY_MAX), fclamp(c.y * GAMMA, PENALTY_MIN, PENALTY_MAX),
                            fclamp(c.z * GAMMA, PENALTY_MIN, PENALTY_MAX), 0.0f);
    float4 pa = make_float4(fclamp(d.x * GAMMA, PENALTY_MIN, PENALTY_MAX), fclamp(d.y * GAMMA, PENALTY_MIN, PENALTY_MAX),
                            fclamp(d.z * GAMMA, PENALTY_MIN, PENALTY_MAX), 0.0f);
    const float K = w.joint_k;
    const uint32_t kind = w.j_kind[j];
    if (K > 0.0f && (kind == AVBD_JOINT_BALL || kind == AVBD_JOINT_REVOLUTE)) {
        // soft rows (anchors and hinge alignment, not the limit) are springs of stiffness K
        pl = make_float4(K, K, K, 0.0f);
        pa.x = K;
        pa.y = K;
    }
    w.j_pen_l[j] = pl;
    w.j_pen_a[j] = pa;
}

void launch_post_discovery(const DW& w, uint32_t* scan_tmp, cudaStream_t st) {
    unsigned gb = nblk(w.N, 256);
    launch_wake_apply(w, st);  // discovery wake votes (rows.rs:938-941)
    launch_wake_joint_motion(w, st);
    k_external_wake<<<gb, 256, 0, st>>>(w);
    unsigned g1 = nblk(w.N + 1, 256);
    k_zero_u32<<<g1, 256, 0, st>>>(w.cnt, w.N + 1);
    k_zero_u32<<<g1, 256, 0, st>>>(w.cur, w.N + 1);
    k_countB<<<gsz(w.pair_cap, 256), 256, 0, st>>>(w);
    scan_exclusive(w.cnt, w.offB, w.N + 1, scan_tmp, st);
    k_placeB<<<gsz(w.pair_cap, 256), 256, 0, st>>>(w);
    k_sortB<<<gb, 256, 0, st>>>(w);
    k_targets<<<gb, 256, 0, st>>>(w);
    k_motion_cache<<<gb, 256, 0, st>>>(w);
    k_decay_points<<<gsz((size_t)w.pair_cap * MAX_PTS, 256), 256, 0, st>>>(w);
    if (w.J) k_decay_joints<<<nblk(w.J, 128), 128, 0, st>>>(w);
}

// ---- colouring --------------------------------------------------------------------
// Jones-Plassmann with hash priorities, one CTA per scene: a body takes the
// smallest colour unused by its neighbours once every higher-priority
// neighbour is coloured.  The result is greedy colouring in descending
// priority, whatever the thread timing, so the CPU oracle reproduces it.
// Vertices: swept bodies; edges: pairs with points and joints between them.
__host__ __device__ __forceinline__ uint32_t colour_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
static __device__ __forceinline__ bool prio_gt(uint32_t la, uint32_t lb) {  // scene-local indices
    uint32_t ha = colour_hash(la), hb = colour_hash(lb);
    return ha != hb ? ha > hb : la > lb;
}
// The colour a pending body takes once every higher-priority neighbour has
// one (the smallest colour none of them uses), or -2 while one is pending.
static __device__ __forceinline__ int jp_pick(const DW& w, volatile int32_t* col, uint32_t h, uint32_t b0) {
    bool ready = true;
    unsigned long long used = 0ull;
    uint32_t lh = h - b0;
    auto visit = [&](uint32_t o) {
        int32_t c = col[o];
        if (c == -2) {
            if (prio_gt(o - b0, lh)) ready = false;
        } else if (c >= 0) {
            used |= 1ull << c;
        }
    };
    for (uint32_t p = w.offA[h]; p < w.offA[h + 1] && ready; p++)
        if (w.p_np[p]) visit(w.p_ab[p].y);
    for (uint32_t k = w.offB[h]; k < w.offB[h + 1] && ready; k++) {
        uint32_t p = w.listB[k];
        if (w.p_np[p]) visit(w.p_ab[p].x);
    }
    for (uint32_t k = w.jofs[h]; k < w.jofs[h + 1] && ready; k++) {
        const uint32_t j = w.jlist[k];
        if (w.j_kind[j] == AVBD_JOINT_GEAR) {  // a gear couples its coupled joints' bodies
            uint32_t m[4];
            const int nm = joint_members(w, j, m);
            for (int i = 0; i < nm; i++)
                if (m[i] != h) visit(m[i]);
            continue;
        }
        uint2 ab = w.j_ab[j];
        visit(ab.x == h ? ab.y : ab.x);
    }
    if (!ready) return -2;
    int c = __ffsll((long long)~used) - 1;
    if (c < 0) {
        atomicOr(&w.ctr[C_ERR], (uint32_t)E_COLOUR_OVERFLOW);
        c = MAX_COLOURS - 1;
    }
    return c;
}
// Scenes above the one-CTA limit: Jones-Plassmann rounds over the whole
// device (a body's colour depends only on its higher-priority neighbours', so
// the rounds give the same colours as the one-CTA loop); the per-scene CTA
// pass afterwards finishes any body still pending.
static __device__ __forceinline__ bool large_scene(const DW& w, uint32_t h, uint32_t small_max, uint32_t& b0) {
    uint32_t s = w.scene_of[h];
    b0 = w.scene_off[s];
    return w.scene_off[s + 1] - b0 > small_max;
}
__global__ void k_colour_init_large(DW w, uint32_t small_max) {
    if (aborted(w)) return;
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < (uint32_t)w.N; h += gridDim.x * blockDim.x) {
        uint32_t b0;
        if (large_scene(w, h, small_max, b0)) w.colour[h] = solved(w, h) ? -2 : -1;
    }
}
__global__ void k_colour_round(DW w, uint32_t small_max) {
    if (aborted(w)) return;
    __shared__ int bmax;
    if (threadIdx.x == 0) bmax = -1;
    __syncthreads();
    volatile int32_t* col = w.colour;
    int maxc = -1;
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < (uint32_t)w.N; h += gridDim.x * blockDim.x) {
        uint32_t b0;
        if (col[h] != -2 || !large_scene(w, h, small_max, b0)) continue;
        int c = jp_pick(w, col, h, b0);
        if (c >= 0) {
            col[h] = c;
            maxc = max(maxc, c);
        }
    }
    if (maxc >= 0) atomicMax(&bmax, maxc);
    __syncthreads();
    if (threadIdx.x == 0 && bmax >= 0) {
        atomicMax(&w.ctr[C_NCOL], (uint32_t)(bmax + 1));
        if (bmax + 1 > w.max_cols) atomicOr(&w.ctr[C_ERR], (uint32_t)E_COLOUR_RANGE);
    }
}
__global__ void __launch_bounds__(1024) k_colour(DW w, uint32_t small_max) {
    if (aborted(w)) return;
    __shared__ int pending;
    uint32_t s = blockIdx.x;
    uint32_t b0 = w.scene_off[s], b1 = w.scene_off[s + 1];
    volatile int32_t* col = w.colour;
    if (b1 - b0 <= small_max)  // large scenes arrive partly coloured by the device-wide rounds
        for (uint32_t h = b0 + threadIdx.x; h < b1; h += blockDim.x) col[h] = solved(w, h) ? -2 : -1;
    __syncthreads();
    int maxc = -1;
    for (uint32_t round = 0; round <= (b1 - b0) + 1; round++) {
        if (threadIdx.x == 0) pending = 0;
        __syncthreads();
        for (uint32_t h = b0 + threadIdx.x; h < b1; h += blockDim.x) {
            if (col[h] != -2) continue;
            int c = jp_pick(w, col, h, b0);
            if (c < 0) {
                pending = 1;
                continue;
            }
            col[h] = c;
            maxc = max(maxc, c);
        }
        __syncthreads();
        if (!pending) break;
        __syncthreads();
    }
    if (maxc >= 0) atomicMax(&w.ctr[C_NCOL], (uint32_t)(maxc + 1));
    if (maxc + 1 > w.max_cols) atomicOr(&w.ctr[C_ERR], (uint32_t)E_COLOUR_RANGE);
}
// Colour lists: one stable 8-bit radix pass over (colour, body) puts the swept
// bodies of each colour in ascending index order (coalesced body loads in
// the primal); uncoloured bodies take digit 255 and sort last.
__global__ void k_colour_keys(DW w, int by_work) {
    if (aborted(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    int c = w.colour[h];
    uint32_t digit = c >= 0 ? (uint32_t)c : 255u;
    uint32_t work = 0;
    if (by_work) {
        // incident pairs: bodies with similar work share a warp in the primal
        work = (w.offA[h + 1] - w.offA[h]) + (w.offB[h + 1] - w.offB[h]);
        work = min(work, 255u);
    }
    w.col_key[h] = (digit << 8) | work;
    w.col_val[h] = h;
}
__global__ void k_colour_starts(DW w, int ntiles) {
    if (aborted(w)) return;
    int c = threadIdx.x;
    if (c <= MAX_COLOURS) w.col_cnt[c] = w.col_hist[(size_t)c * ntiles];
}
void launch_colouring(const DW& w, const Tune& tune, uint32_t* scan_tmp, cudaStream_t st) {
    const uint32_t small_max = (uint32_t)tune.small_scene_max;
    if (w.n_large_scenes) {
        k_colour_init_large<<<gsz(w.N, 256), 256, 0, st>>>(w, small_max);
        for (int r = 0; r < COLOUR_ROUNDS; r++) k_colour_round<<<gsz(w.N, 256), 256, 0, st>>>(w, small_max);
    }
    k_colour<<<w.S, 1024, 0, st>>>(w, small_max);
    k_colour_keys<<<nblk(w.N, 256), 256, 0, st>>>(w, tune.sort_work);
    int ntiles;
    if (tune.sort_work) {
        // LSD: work byte, then colour byte (stable: index order within equal work)
        radix_pass(w.col_key, w.col_val, w.col_key2, w.col_list, (size_t)w.N, 0, w.col_hist, scan_tmp, st);
        ntiles = radix_pass(w.col_key2, w.col_list, w.col_key, w.col_val, (size_t)w.N, 8, w.col_hist, scan_tmp, st);
        cudaMemcpyAsync(w.col_list, w.col_val, (size_t)w.N * 4, cudaMemcpyDeviceToDevice, st);
    } else {
        ntiles = radix_pass(w.col_key, w.col_val, w.col_key2, w.col_list, (size_t)w.N, 8, w.col_hist, scan_tmp, st);
    }
    k_colour_starts<<<1, 128, 0, st>>>(w, ntiles);
}

}  // namespace avbd
