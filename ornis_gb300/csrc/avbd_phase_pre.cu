// avbd_phase_pre.cu — substep prologue: wake bookkeeping, torque, broadphase
// (sweep-and-prune) and the linear CCD clamp.
//
// Reference: crates/physics/src/avbd/mod.rs:846-978, avbd/sleep.rs:107-137,
// avbd/rows.rs:253-292 (bounding radii), :767-793 (the O(n^2) sphere
// prefilter this broadphase replaces), collision/distance.rs:841-893
// (cast_shape).
#include "avbd_common.cuh"

namespace avbd {

__global__ void k_begin(DW w) {
    if (threadIdx.x == 0) {
        w.ctr[C_CCD_PENDING] = 0;
        w.ctr[C_BOXPAIRS] = 0;
        w.ctr[C_FCAND] = 0;
        w.ctr[C_BOXONE] = 0;
        w.ctr[C_NOBOX] = 0;
        w.ctr[C_LONGSEG] = 0;
        w.ctr[C_CAND] = 0;
        w.ctr[C_NCOL] = 0;
        w.ctr[C_FAST] = 0;
        w.ctr[C_POINTS] = 0;
        w.ctr[C_SLEEP] = 0;
        w.ctr[C_CCD_HITS] = 0;
        if (w.evs) w.evs[EV_TRIG_NOW] = 0;
    }
}
void launch_begin_substep(const DW& w, cudaStream_t st) { k_begin<<<1, 32, 0, st>>>(w); }

// ---- wake_joint_motion (sleep.rs:107-137) ----------------------------------
__global__ void k_wake_flags(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    uint8_t f = 0;
    if (is_dynamic(w, h)) {
        float4 v = w.vel[h], om = w.angvel[h], tq = w.torque[h];
        float4 p = w.pos[h], pp = w.prev_pos[h], q = w.rot[h], pq = w.prev_rot[h];
        f = !w.asleep[h] || v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || om.x != 0.0f || om.y != 0.0f ||
            om.z != 0.0f || tq.x != 0.0f || tq.y != 0.0f || tq.z != 0.0f || p.x != pp.x || p.y != pp.y ||
            p.z != pp.z || q.x != pq.x || q.y != pq.y || q.z != pq.z || q.w != pq.w;
    }
    w.flag[h] = f;
}
__global__ void k_joint_wake(DW w) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (uint32_t)w.J) return;
    if (joint_driven(w, j) || joint_rest_error(w, j) > JOINT_REST_ERROR) {
        uint32_t m[4];
        const int nm = joint_members(w, j, m);
        for (int k = 0; k < nm; k++)
            if (is_dynamic(w, m[k])) w.flag[m[k]] = 1;
    }
}
// propagate_joint_flags (sleep.rs:152-175) with value 1: one awake dynamic
// member wakes its whole joint component (components precomputed on the host)
__global__ void k_comp_gather_set(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    int c = w.comp[h];
    if (c >= 0 && is_dynamic(w, h) && w.flag[h] == 1) w.comp_flag[c] = 1;
}
__global__ void k_comp_scatter_set(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    int c = w.comp[h];
    if (c >= 0 && is_dynamic(w, h) && w.comp_flag[c]) w.flag[h] = 1;
}
__global__ void k_wake_apply(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    if (w.flag[h] && w.asleep[h]) wake_body(w, h);
}
void launch_wake_joint_motion(const DW& w, cudaStream_t st) {
    unsigned gb = nblk(w.N, 256);
    k_wake_flags<<<gb, 256, 0, st>>>(w);
    if (w.J) {
        k_joint_wake<<<nblk(w.J, 128), 128, 0, st>>>(w);
        k_comp_clear<<<gb, 256, 0, st>>>(w);
        k_comp_gather_set<<<gb, 256, 0, st>>>(w);
        k_comp_scatter_set<<<gb, 256, 0, st>>>(w);
    }
    k_wake_apply<<<gb, 256, 0, st>>>(w);
}
void launch_wake_apply(const DW& w, cudaStream_t st) { k_wake_apply<<<nblk(w.N, 256), 256, 0, st>>>(w); }

// Once per step, after the first wake pass: each gear's coupled joints'
// raw coordinates and the continuous ones, unwrapped across turns for
// hinges (update_gear_mem, joints_ext.rs:55-118).
__global__ void k_gear_mem(DW w) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (uint32_t)w.J || w.j_kind[g] != AVBD_JOINT_GEAR) return;
    const uint2 gb = w.j_gb[g];
    const float4 m = w.j_gmem[g];
    const bool set = w.j_gset[g] != 0u;
    GearSide sa, sb;
    const float ra = joint_coordinate(w, gb.x, &sa), rb = joint_coordinate(w, gb.y, &sb);
    const float ca = set && sa.angular ? m.z + wrap_pi(ra - m.x) : ra;
    const float cb = set && sb.angular ? m.w + wrap_pi(rb - m.y) : rb;
    w.j_gmem[g] = make_float4(ra, rb, ca, cb);
    w.j_gset[g] = 1u;
}
void launch_gear_mem(const DW& w, cudaStream_t st) {
    if (w.n_gear) k_gear_mem<<<nblk(w.J, 128), 128, 0, st>>>(w);
}

// ---- torque -> angular velocity (mod.rs:855-871) ---------------------------
__global__ void k_torque(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    if (w.pre_vel) w.pre_vel[h] = w.vel[h];  // torque leaves the linear velocity as it is
    if (!solvable(w, h)) return;
    float4 tq4 = w.torque[h];
    V3 in = ld3(w.inertia[h]);
    float iw[3][3], inv[3][3];
    world_inertia(in, ldq(w.rot[h]), iw);
    V3 dg{in.x > 0.0f ? in.x : 0.0f, in.y > 0.0f ? in.y : 0.0f, in.z > 0.0f ? in.z : 0.0f};
    inverse_symmetric(iw, dg, inv);
    w.torque[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    V3 om = ld3(w.angvel[h]) + mat3_vec(inv, ld3(tq4)) * w.dt;
    w.angvel[h] = st3(om, 0.0f);
}

// ---- motor and rope impulses (mod.rs:872-873, joints_ext.rs:173-420) ---------
// Deadbeat velocity impulses of velocity motors (revolute, prismatic) and of
// stretched ropes, after the torque and before the warm start.  The
// reference applies them joint by joint in order (each sees the velocities
// the earlier ones left), so one thread per scene walks that scene's motor
// and rope joints in joint order: all motors, then all ropes.
static __device__ V3 ang_inv_wa(const DW& w, uint32_t h, V3 wa) {  // joints_ext.rs:423-437
    if (!solvable(w, h)) return V0();
    V3 in = ld3(w.inertia[h]);
    float iw[3][3], inv[3][3];
    world_inertia(in, ldq(w.rot[h]), iw);
    V3 dg{fmaxf(in.x, 0.0f), fmaxf(in.y, 0.0f), fmaxf(in.z, 0.0f)};
    inverse_symmetric(iw, dg, inv);
    return mat3_vec(inv, wa);
}
// JointMotor::velocity_impulse (joint.rs:1172-1177)
static __device__ __forceinline__ float velocity_impulse(const DW& w, float rate_error, float inv_eff, float max_f) {
    if (!(w.dt > 0.0f) || max_f <= 0.0f || inv_eff <= 0.0f) return 0.0f;
    return fclamp(rate_error / inv_eff, -max_f * w.dt, max_f * w.dt);
}
static __device__ bool limit_violated(const DW& w, uint32_t j) {  // joints_ext.rs:441-462
    float4 lim = w.j_lim[j];
    if (lim.z == 0.0f) return false;
    uint2 ab = w.j_ab[j];
    Q qa = ldq(w.rot[ab.x]), qb = ldq(w.rot[ab.y]);
    float4 axa4 = w.j_axa[j];
    if (w.j_kind[j] == AVBD_JOINT_REVOLUTE) {
        float angle = wrap_pi(hinge_twist(qa, qb, ld3(axa4)) - axa4.w);
        return limit_state(angle, lim.x, lim.y, LIMIT_SLOP_ANG) >= 0;
    }
    if (w.j_kind[j] == AVBD_JOINT_PRISMATIC) {
        V3 wa = normalize_or(qrot(qa, ld3(axa4)), VZ());
        V3 pa = ld3(w.pos[ab.x]) + qrot(qa, ld3(w.j_la[j])), pb = ld3(w.pos[ab.y]) + qrot(qb, ld3(w.j_lb[j]));
        return limit_state(dot(pb - pa, wa) - w.j_ref[j].x, lim.x, lim.y, LIMIT_SLOP_LIN) >= 0;
    }
    return false;
}
// free_motor_impulse (joints_ext.rs:384-420): per world axis, the deadbeat
// linear then angular drive of B relative to A (MotorDrive's impulses,
// joint.rs:485-499, are velocity_impulse's formula)
static __device__ void free_motor_impulse(const DW& w, uint32_t j) {
    const uint2 ab = w.j_ab[j];
    const uint32_t a = ab.x, b = ab.y;
    const V3 lin = ld3(w.j_axa[j]), ang = ld3(w.j_axb[j]);
    const float4 ref = w.j_ref[j];
    for (int i = 0; i < 3; i++) {
        V3 axis = V0();
        axis[i] = 1.0f;
        float v = dot(ld3(w.vel[b]) - ld3(w.vel[a]), axis);
        float ka = eff_inv_mass(w, a), kb = eff_inv_mass(w, b);
        float dj = velocity_impulse(w, dot(lin, axis) - v, ka + kb, ref.z);
        if (dj != 0.0f) {
            if (solvable(w, a)) w.vel[a] = st3(ld3(w.vel[a]) + axis * (-dj * ka), 0.0f);
            if (solvable(w, b)) w.vel[b] = st3(ld3(w.vel[b]) + axis * (dj * kb), 0.0f);
        }
        float om = dot(ld3(w.angvel[b]) - ld3(w.angvel[a]), axis);
        V3 ia = ang_inv_wa(w, a, axis), ib = ang_inv_wa(w, b, axis);
        float k = dot(ia, axis) + dot(ib, axis);
        float dw = velocity_impulse(w, dot(ang, axis) - om, k, ref.w);
        if (dw != 0.0f) {
            if (solvable(w, a)) w.angvel[a] = st3(ld3(w.angvel[a]) + (-dw) * ia, 0.0f);
            if (solvable(w, b)) w.angvel[b] = st3(ld3(w.angvel[b]) + dw * ib, 0.0f);
        }
    }
}
static __device__ void motor_impulse(const DW& w, uint32_t j) {  // joints_ext.rs:237-383
    if (w.j_kind[j] == AVBD_JOINT_MOTOR) {  // free motors carry their drive inline
        free_motor_impulse(w, j);
        return;
    }
    float4 ref = w.j_ref[j];
    if (!(ref.w > 0.0f) || limit_violated(w, j)) return;
    uint2 ab = w.j_ab[j];
    const uint32_t a = ab.x, b = ab.y;
    V3 wa = normalize_or(qrot(ldq(w.rot[a]), ld3(w.j_axa[j])), VZ());
    if (w.j_kind[j] == AVBD_JOINT_REVOLUTE) {
        float om = dot(ld3(w.angvel[b]) - ld3(w.angvel[a]), wa);
        V3 ia = ang_inv_wa(w, a, wa), ib = ang_inv_wa(w, b, wa);
        float k = dot(ia, wa) + dot(ib, wa);
        if (k < MIN_EFFECTIVE_MASS) return;
        float dj = velocity_impulse(w, ref.z - om, k, ref.w);
        if (solvable(w, a)) w.angvel[a] = st3(ld3(w.angvel[a]) + (-dj) * ia, 0.0f);
        if (solvable(w, b)) w.angvel[b] = st3(ld3(w.angvel[b]) + dj * ib, 0.0f);
    } else if (w.j_kind[j] == AVBD_JOINT_WHEEL) {  // spin about the axle (joints_ext.rs:337-371)
        V3 xa = normalize_or(qrot(ldq(w.rot[a]), ld3(w.j_dref[j])), VZ());
        float om = dot(ld3(w.angvel[b]) - ld3(w.angvel[a]), xa);
        V3 ia = ang_inv_wa(w, a, xa), ib = ang_inv_wa(w, b, xa);
        float k = dot(ia, xa) + dot(ib, xa);
        if (k < MIN_EFFECTIVE_MASS) return;
        float dj = velocity_impulse(w, ref.z - om, k, ref.w);
        if (solvable(w, a)) w.angvel[a] = st3(ld3(w.angvel[a]) + (-dj) * ia, 0.0f);
        if (solvable(w, b)) w.angvel[b] = st3(ld3(w.angvel[b]) + dj * ib, 0.0f);
    } else if (w.j_kind[j] == AVBD_JOINT_PRISMATIC) {
        float v = dot(ld3(w.vel[b]) - ld3(w.vel[a]), wa);
        float ka = eff_inv_mass(w, a), kb = eff_inv_mass(w, b);
        float k = ka + kb;
        if (k < MIN_EFFECTIVE_MASS) return;
        float dj = velocity_impulse(w, ref.z - v, k, ref.w);
        if (solvable(w, a)) w.vel[a] = st3(ld3(w.vel[a]) + (-dj) * ka * wa, 0.0f);
        if (solvable(w, b)) w.vel[b] = st3(ld3(w.vel[b]) + dj * kb * wa, 0.0f);
    }
}
static __device__ void rope_impulse(const DW& w, uint32_t j) {  // joints_ext.rs:173-236
    uint2 ab = w.j_ab[j];
    const uint32_t a = ab.x, b = ab.y;
    V3 xa = ld3(w.pos[a]), xb = ld3(w.pos[b]);
    V3 pa = xa + qrot(ldq(w.rot[a]), ld3(w.j_la[j])), pb = xb + qrot(ldq(w.rot[b]), ld3(w.j_lb[j]));
    V3 delta = pb - pa;
    float ln = len(delta);
    if (ln <= w.j_ref[j].x) return;
    V3 n = delta / ln;
    V3 ra = pa - xa, rb = pb - xb;
    float ka = eff_inv_mass(w, a), kb = eff_inv_mass(w, b);
    V3 ta = cross(ra, n), tb = cross(rb, n);
    float k = ka + kb + dot(ang_inv_wa(w, a, ta), ta) + dot(ang_inv_wa(w, b, tb), tb);
    if (k < MIN_EFFECTIVE_MASS) return;
    V3 va = ld3(w.vel[a]) + cross(ld3(w.angvel[a]), ra);
    V3 vb = ld3(w.vel[b]) + cross(ld3(w.angvel[b]), rb);
    float vsep = dot(vb - va, n);
    if (vsep <= 0.0f) return;
    float dj = -vsep / k;
    if (solvable(w, a)) {
        V3 ia = ang_inv_wa(w, a, ta);
        w.vel[a] = st3(ld3(w.vel[a]) - n * (dj * ka), 0.0f);
        w.angvel[a] = st3(ld3(w.angvel[a]) - ia * dj, 0.0f);
    }
    if (solvable(w, b)) {
        V3 ib = ang_inv_wa(w, b, tb);
        w.vel[b] = st3(ld3(w.vel[b]) + n * (dj * kb), 0.0f);
        w.angvel[b] = st3(ld3(w.angvel[b]) + ib * dj, 0.0f);
    }
}
__global__ void k_joint_impulses(DW w) {
    uint32_t sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= (uint32_t)w.S) return;
    const uint32_t k0 = w.jimp_off[sc], k1 = w.jimp_off[sc + 1];
    for (uint32_t k = k0; k < k1; k++) motor_impulse(w, w.jimp_list[k]);
    for (uint32_t k = k0; k < k1; k++)
        if (w.j_kind[w.jimp_list[k]] == AVBD_JOINT_ROPE) rope_impulse(w, w.jimp_list[k]);
    if (w.pre_vel)  // the velocity snapshot is taken after the impulses (mod.rs:874-876)
        for (uint32_t k = k0; k < k1; k++) {
            uint2 ab = w.j_ab[w.jimp_list[k]];
            w.pre_vel[ab.x] = w.vel[ab.x];
            w.pre_vel[ab.y] = w.vel[ab.y];
        }
}
void launch_torque(const DW& w, cudaStream_t st) {
    k_torque<<<nblk(w.N, 256), 256, 0, st>>>(w);
    if (w.n_imp) k_joint_impulses<<<nblk(w.S, 64), 64, 0, st>>>(w);
}

// ---- broadphase ---------------------------------------------------------------
// shape_min_dimension (rows.rs:373-403)
static __device__ __forceinline__ float min_dim(const DW& w, uint32_t kind, float4 sp) {
    if (kind == AVBD_SHAPE_SPHERE) return sp.x;
    if (kind == AVBD_SHAPE_BOX) return fminf(sp.x, fminf(sp.y, sp.z));
    if (kind == AVBD_SHAPE_CAPSULE) return sp.x;
    if (kind == AVBD_SHAPE_CYLINDER) return fminf(sp.x, sp.y);
    if (kind == AVBD_SHAPE_CONE) return HALF * fminf(sp.x, sp.y);
    if (kind == AVBD_SHAPE_HULL) {
        uint32_t id = (uint32_t)sp.x;
        return HALF * (id < w.nhulls ? w.hulls[id].min_ext : 0.0f);
    }
    if (ext_kind(kind)) return w.exts[(uint32_t)sp.x].min_dim;
    if (kind == AVBD_SHAPE_HEIGHTFIELD) return HALF * w.hfs[(uint32_t)sp.x].cell;
    if (kind == AVBD_SHAPE_TRIMESH) return HALF * w.meshes[(uint32_t)sp.x].min_feature;
    return INFINITY;
}
// CCD mover gate (mod.rs:882-895): returns the step travel |v h| of a body
// that sweeps, 0 for every other body.
static __device__ __forceinline__ float ccd_travel(const DW& w, uint32_t h) {
    if (!w.enable_ccd || !solvable(w, h) || w.asleep[h] || info_trigger(w.info[h])) return 0.0f;
    V3 disp = ld3(w.vel[h]) * w.dt;
    float l = len(disp);
    if (l <= CCD_TRAVEL_GATE_FRACTION * min_dim(w, info_shape(w.info[h]), w.shp[h])) return 0.0f;
    if (l < NEAR_ZERO) return 0.0f;
    return l;
}

// Cube around the bounding sphere grown by half the creation margin and by
// the CCD travel: every pair the sphere prefilter (rows.rs:475-479) can accept,
// before or after the CCD clamp, and every pair a TOI sweep can hit, has
// overlapping cubes.
__global__ void k_aabb(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    float travel = ccd_travel(w, h);
    w.fast[h] = travel > 0.0f;
    float e = w.shp[h].w + HALF * GEN_MARGIN + travel;
    e = e * 1.0001f + 1e-4f;  // outward slack for the rounding of this sum
    float4 p = w.pos[h];
    w.aabb_lo[h] = make_float4(p.x - e, p.y - e, p.z - e, 0.0f);
    w.aabb_hi[h] = make_float4(p.x + e, p.y + e, p.z + e, 0.0f);
}

static __device__ __forceinline__ void emit_candidate(const DW& w, uint32_t a, uint32_t b) {
    uint32_t lo = min(a, b), hi = max(a, b);
    uint32_t slot = agg_inc(&w.ctr[C_CAND]);
    if (slot < w.cand_cap) w.cand[slot] = make_uint2(lo, hi);
    else atomicOr(&w.ctr[C_ERR], (uint32_t)E_CAND_OVERFLOW);
}
static __device__ __forceinline__ bool overlap_yz(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    return alo.y <= bhi.y && blo.y <= ahi.y && alo.z <= bhi.z && blo.z <= ahi.z;
}

// One CTA per small scene: bitonic sort of (min-x key, body) in shared
// memory, then each thread sweeps forward from its sorted slot.
constexpr int SAP_SMALL = 2048;
__global__ void __launch_bounds__(512) k_sap_small(DW w, const uint32_t* scenes, int nscenes) {
    __shared__ unsigned long long kv[SAP_SMALL];
    __shared__ int cnt;
    int si = blockIdx.x;
    if (si >= nscenes) return;
    uint32_t s = scenes[si];
    uint32_t b0 = w.scene_off[s], b1 = w.scene_off[s + 1];
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    for (uint32_t h = b0 + threadIdx.x; h < b1; h += blockDim.x) {
        if (unbounded_kind(info_shape(w.info[h]))) continue;
        int k = atomicAdd(&cnt, 1);
        kv[k] = ((unsigned long long)f2key(w.aabb_lo[h].x) << 32) | h;
    }
    __syncthreads();
    int n = cnt;
    int m = 1;
    while (m < n) m <<= 1;
    for (int i = n + threadIdx.x; i < m; i += blockDim.x) kv[i] = ~0ull;
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                int ixj = i ^ j;
                if (ixj > i) {
                    unsigned long long x = kv[i], y = kv[ixj];
                    bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        kv[i] = y;
                        kv[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t a = (uint32_t)(kv[i] & 0xffffffffu);
        float4 alo = w.aabb_lo[a], ahi = w.aabb_hi[a];
        for (int j = i + 1; j < n; j++) {
            uint32_t b = (uint32_t)(kv[j] & 0xffffffffu);
            float4 blo = w.aabb_lo[b];
            if (blo.x > ahi.x) break;
            if (overlap_yz(alo, ahi, blo, w.aabb_hi[b])) emit_candidate(w, a, b);
        }
    }
}

// Large scenes: device-wide radix sort of the scene's min-x keys (half-space
// bodies get the largest key and end every sweep), then one thread per
// sorted slot sweeps forward.
__global__ void k_sap_keys(DW w, uint32_t b0, uint32_t b1) {
    uint32_t h = b0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= b1) return;
    bool plane = unbounded_kind(info_shape(w.info[h]));
    w.sort_key[h - b0] = plane ? 0xffffffffu : f2key(w.aabb_lo[h].x);
    w.sort_idx[h - b0] = h;
}
__global__ void k_sap_sweep(DW w, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t a = w.sort_idx[i];
    if (unbounded_kind(info_shape(w.info[a]))) return;
    float4 alo = w.aabb_lo[a], ahi = w.aabb_hi[a];
    for (uint32_t j = i + 1; j < n; j++) {
        uint32_t b = w.sort_idx[j];
        if (unbounded_kind(info_shape(w.info[b]))) break;
        float4 blo = w.aabb_lo[b];
        if (blo.x > ahi.x) break;
        if (overlap_yz(alo, ahi, blo, w.aabb_hi[b])) emit_candidate(w, a, b);
    }
}
// Large scenes, cell rows: space is cut into cells at least as wide as the
// scene's widest AABB (so overlapping boxes have centres in the same or
// adjacent cells along every axis); a row is the cells of one (y, z) cell
// pair, all x.  Bodies are sorted by (row Morton code, min x) with two
// stable radix sorts; each body sweeps its own row forward in x as the
// one-axis sweep does, and the four rows of the forward half of its (y, z)
// neighbourhood over the x window its box can reach.  Every overlapping pair
// is tested exactly once, with the same closed-interval test: the candidate
// set is the one-axis sweep's.  Cell coordinates are taken in double from
// the boxes' float bounds, with a 1% wider cell, so that rounding cannot
// move a pair more than one cell apart.
__device__ __forceinline__ uint32_t part1by1(uint32_t x) {
    x &= 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}
// Cell coordinate of a centre: floor(c / cell) shifted into [0, 65534]
// (clamping keeps adjacent cells adjacent; 65535 would collide with the
// half-space key).
__device__ __forceinline__ int cell_of(double c, double cell) {
    double k = floor(c / cell) + 32768.0;
    return (int)fmin(fmax(k, 0.0), 65534.0);
}
__device__ __forceinline__ uint32_t row_code(int cy, int cz) { return (part1by1(cy) << 1) | part1by1(cz); }
__device__ __forceinline__ double row_cell(float wmax) { return 1.01 * (double)wmax; }
__device__ __forceinline__ void row_cells(const DW& w, uint32_t h, double cell, int& cy, int& cz) {
    float4 lo = w.aabb_lo[h], hi = w.aabb_hi[h];
    cy = cell_of(0.5 * ((double)lo.y + (double)hi.y), cell);
    cz = cell_of(0.5 * ((double)lo.z + (double)hi.z), cell);
}
// the scene's widest AABB edge (boxes are cubes here; every axis is taken)
__global__ void k_sap_extent(DW w, uint32_t b0, uint32_t b1, float* ext) {
    float m = 0.0f;
    for (uint32_t h = b0 + blockIdx.x * blockDim.x + threadIdx.x; h < b1; h += gridDim.x * blockDim.x) {
        if (unbounded_kind(info_shape(w.info[h]))) continue;
        float4 lo = w.aabb_lo[h], hi = w.aabb_hi[h];
        m = fmaxf(m, fmaxf(hi.x - lo.x, fmaxf(hi.y - lo.y, hi.z - lo.z)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax((int*)ext, __float_as_int(m));  // m >= 0: int order
}
__global__ void k_sap_row_keys(DW w, uint32_t b0, uint32_t b1, const float* ext, uint32_t* row_key) {
    uint32_t h = b0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= b1) return;
    bool plane = unbounded_kind(info_shape(w.info[h]));
    uint32_t rk = 0xffffffffu;
    if (!plane) {
        int cy, cz;
        row_cells(w, h, row_cell(*ext), cy, cz);
        rk = row_code(cy, cz);
    }
    w.sort_key[h - b0] = plane ? 0xffffffffu : f2key(w.aabb_lo[h].x);
    w.sort_idx[h - b0] = h;
    row_key[h - b0] = rk;
}
// after the sort by min x: the row codes in that order (the second sort's keys)
__global__ void k_sap_row_gather(DW w, uint32_t b0, uint32_t n, const uint32_t* row_key) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w.sort_key[i] = row_key[w.sort_idx[i] - b0];
}
// first sorted slot in [lo, hi) whose row code is >= key
__device__ __forceinline__ uint32_t row_lower(const uint32_t* keys, uint32_t lo, uint32_t hi, uint32_t key) {
    while (lo < hi) {
        uint32_t m = (lo + hi) >> 1;
        if (keys[m] < key) lo = m + 1;
        else hi = m;
    }
    return lo;
}
__global__ void k_sap_row_sweep(DW w, uint32_t n, const float* ext) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t rk = w.sort_key[i];
    if (rk == 0xffffffffu) return;  // half-spaces sort last
    const uint32_t a = w.sort_idx[i];
    const float4 alo = w.aabb_lo[a], ahi = w.aabb_hi[a];
    for (uint32_t j = i + 1; j < n && w.sort_key[j] == rk; j++) {
        uint32_t b = w.sort_idx[j];
        float4 blo = w.aabb_lo[b];
        if (blo.x > ahi.x) break;
        if (overlap_yz(alo, ahi, blo, w.aabb_hi[b])) emit_candidate(w, a, b);
    }
    const float wmax = *ext;
    int cy, cz;
    row_cells(w, a, row_cell(wmax), cy, cz);
    // a neighbour's box reaches x >= alo.x only if its min x is at least this
    const double reach = (double)alo.x - 1.01 * (double)wmax - 1e-6 * fabs((double)alo.x);
    const int dy[4] = {0, 1, 1, 1}, dz[4] = {1, -1, 0, 1};
    for (int k = 0; k < 4; k++) {
        int ny = cy + dy[k], nz = cz + dz[k];
        if (ny > 65534 || nz < 0 || nz > 65534) continue;
        const uint32_t nk = row_code(ny, nz);
        uint32_t r0 = row_lower(w.sort_key, 0, n, nk);
        uint32_t r1 = row_lower(w.sort_key, r0, n, nk + 1u);
        // first slot of the row whose min x reaches the window
        uint32_t lo = r0, hi = r1;
        while (lo < hi) {
            uint32_t m = (lo + hi) >> 1;
            if ((double)w.aabb_lo[w.sort_idx[m]].x < reach) lo = m + 1;
            else hi = m;
        }
        for (uint32_t j = lo; j < r1; j++) {
            uint32_t b = w.sort_idx[j];
            float4 blo = w.aabb_lo[b];
            if (blo.x > ahi.x) break;
            float4 bhi = w.aabb_hi[b];
            if (alo.x <= bhi.x && overlap_yz(alo, ahi, blo, bhi)) emit_candidate(w, a, b);
        }
    }
}

// Half-space bodies have an unbounded prefilter radius (rows.rs:290), so the
// reference narrowphases every (plane, body) pair.  A pair can only survive
// discovery if it already exists (an empty shell is kept) or if the body can
// come within the creation reach of the plane this substep; the body's
// support distance is at least (x - p).n - bound_radius, its approach at most
// |v_b| + |v_p| (twice that after a CCD bounce), and a CCD clamp moves it by at
// most its travel.  Pairs outside that conservative reach are not emitted.
__global__ void k_plane_cands(DW w) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    // an unbounded body pairs with the unbounded bodies listed before it
    // (each such pair once; they meet as separation or a static shell)
    const uint32_t kh = info_shape(w.info[h]);
    const bool unb = unbounded_kind(kh);
    uint32_t s = w.scene_of[h];
    V3 x = ld3(w.pos[h]);
    float vh = len(ld3(w.vel[h]));
    float travel = ccd_travel(w, h);
    float rb = w.shp[h].w;
    for (uint32_t k = w.plane_off[s]; k < w.plane_off[s + 1]; k++) {
        uint32_t pl = w.plane_list[k];
        if (unb && pl >= h) break;  // listed in ascending handle order
        // two half-spaces never meet (distance.rs:619-621): not a candidate
        if (kh == AVBD_SHAPE_HALFSPACE && info_shape(w.info[pl]) == AVBD_SHAPE_HALFSPACE) continue;
        // terrain and meshes: no bound to prune by (rows.rs:274)
        if (info_shape(w.info[pl]) == AVBD_SHAPE_HALFSPACE && find_old_pair(w, min(pl, h), max(pl, h)) < 0) {
            float4 sp = w.shp[pl];
            V3 n = qrot(ldq(w.rot[pl]), V3{sp.x, sp.y, sp.z});
            float dlow = dot(x - ld3(w.pos[pl]), n) - rb;
            float reach = GEN_MARGIN + 2.0f * (vh + len(ld3(w.vel[pl]))) * w.dt + travel;
            if (dlow > reach + 1e-3f + 1e-5f * fabsf(dlow)) continue;
        }
        emit_candidate(w, pl, h);
    }
}

void launch_broadphase(const DW& w, const BroadphasePlan& plan, cudaStream_t st) {
    k_aabb<<<nblk(w.N, 256), 256, 0, st>>>(w);
    k_plane_cands<<<nblk(w.N, 256), 256, 0, st>>>(w);
    if (plan.n_small) k_sap_small<<<plan.n_small, 512, 0, st>>>(w, plan.small_scenes, plan.n_small);
    for (size_t i = 0; i < plan.large.size(); i++) {
        uint32_t b0 = plan.large[i].first, b1 = plan.large[i].second;
        uint32_t n = b1 - b0;
        if (plan.rows) {
            float* ext = plan.ext + i;
            cudaMemsetAsync(ext, 0, sizeof(float), st);
            k_sap_extent<<<std::min<unsigned>(nblk(n, 256), 4u * 152u), 256, 0, st>>>(w, b0, b1, ext);
            k_sap_row_keys<<<nblk(n, 256), 256, 0, st>>>(w, b0, b1, ext, plan.row_key);
            radix_sort_pairs(w.sort_key, w.sort_idx, plan.keys_alt, plan.vals_alt, n, plan.hist, plan.scan_tmp, st);
            k_sap_row_gather<<<nblk(n, 256), 256, 0, st>>>(w, b0, n, plan.row_key);
            radix_sort_pairs(w.sort_key, w.sort_idx, plan.keys_alt, plan.vals_alt, n, plan.hist, plan.scan_tmp, st);
            k_sap_row_sweep<<<nblk(n, 128), 128, 0, st>>>(w, n, ext);
            continue;
        }
        k_sap_keys<<<nblk(n, 256), 256, 0, st>>>(w, b0, b1);
        radix_sort_pairs(w.sort_key, w.sort_idx, plan.keys_alt, plan.vals_alt, n, plan.hist, plan.scan_tmp, st);
        k_sap_sweep<<<nblk(n, 128), 128, 0, st>>>(w, n);
    }
}

// ---- CCD (mod.rs:882-978, distance.rs:841-893) -------------------------------
// The reference clamps movers one at a time in handle order, each sweep
// seeing the already-clamped poses of earlier movers.  Here every mover casts
// in parallel; a mover whose candidate targets include an earlier mover waits
// for it (dependency rounds), and recasts if that mover actually moved — the
// same poses the serial loop would have seen.
struct Cast {
    bool hit;
    float t;
    V3 normal;
    V3 point;  // the target's witness at the hit
};
static __device__ __noinline__ Cast cast_one(const DW& w, uint32_t h, uint32_t o) {
    Cast c{false, 0.0f, V0(), V0()};
    V3 disp = ld3(w.vel[h]) * w.dt;
    float L = len(disp);
    if (L < NEAR_ZERO) return c;
    V3 dir = disp / L;
    Shape mv = shape_of(w, h);
    Shape tg = shape_of(w, o);
    V3 p0 = mv.pos;
    float t = 0.0f;
    for (int it = 0; it < 24; it++) {
        mv.pos = p0 + dir * t;
        Dist d = ext_distance(w, mv, tg, nullptr);
        if (d.dist <= SHAPE_TOUCH) {
            if (t > 0.0f) {
                c.hit = true;
                c.t = t;
                c.normal = normalize_or(d.pa - d.pb, -dir);
                c.point = d.pb;
            }
            break;
        }
        t += d.dist - SHAPE_TOUCH * HALF;
        if (t >= L) break;
    }
    return c;
}
static __device__ __forceinline__ bool ccd_target(const DW& w, uint32_t h, uint32_t o) {
    return !info_trigger(w.info[o]) && pair_allowed(w, h, o) && !jointed(w, h, o);
}
// Whether the sweep of h along its step displacement can bring it within
// touching distance of o: its bounding sphere swept along the segment
// against o's bounding sphere (or o's plane).  When it cannot, cast_one
// returns no hit (every distance it evaluates exceeds SHAPE_TOUCH), so the
// cast is skipped; the slack covers the float rounding of both tests.
static __device__ __forceinline__ bool sweep_may_touch(const DW& w, uint32_t h, uint32_t o) {
    const V3 p0 = ld3(w.pos[h]), d = ld3(w.vel[h]) * w.dt, c = ld3(w.pos[o]);
    const float rh = w.shp[h].w;
    const float slack = 4.0f * SHAPE_TOUCH + 1e-4f * (len(p0) + len(c) + len(d));
    if (!isfinite(rh)) return true;
    if (info_shape(w.info[o]) == AVBD_SHAPE_HALFSPACE) {
        const float4 sp = w.shp[o];
        const V3 n = qrot(ldq(w.rot[o]), V3{sp.x, sp.y, sp.z});
        const float d0 = dot(p0 - c, n), d1 = d0 + dot(d, n);
        return fminf(d0, d1) - rh <= slack;
    }
    const float ro = w.shp[o].w;
    if (!isfinite(ro)) return true;
    const float dd = dot(d, d);
    const float sp = dd > 0.0f ? fclamp(dot(c - p0, d) / dd, 0.0f, 1.0f) : 0.0f;
    return len(c - (p0 + d * sp)) - rh - ro <= slack;
}
__global__ void k_ccd_init(DW w) {
    if (aborted(w)) return;
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= (uint32_t)w.N) return;
    w.ccd_best[h] = ~0ull;
    if (w.ccd_win) w.ccd_win[h] = ~0u;
    if (w.ccd_ev_o) w.ccd_ev_o[h] = -1;
    w.ccd_deps[h] = 0;
    w.ccd_state[h] = 0;
    w.ccd_recompute[h] = 0;
    if (w.sort_static) w.ccd_rec[2 * h + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (w.fast[h]) {
        w.fbody[agg_inc(&w.ctr[C_FAST])] = h;
        agg_inc(&w.ctr[C_CCD_PENDING]);
    }
}
// first = 1: every mover casts against its candidates at the step-top poses
// and counts the earlier movers among its targets.  first = 0: only movers
// flagged for a recast.  Every hit is recorded (tag = the cast round) so
// that the apply can take the winner's time, normal and witness instead of
// casting again: the winner's inputs do not change between its cast and its
// apply (a mover applies once its earlier movers are final and it has recast
// against any that moved; later movers wait for it).
static __device__ __forceinline__ void k_ccd_cast_one(const DW& w, int first, uint32_t c, uint32_t tag) {
    uint2 ab = w.cand[c];
    bool fa = w.fast[ab.x], fb = w.fast[ab.y];
    if (!fa && !fb) return;
    for (int k = 0; k < 2; k++) {
        uint32_t h = k ? ab.y : ab.x, o = k ? ab.x : ab.y;
        if (!(k ? fb : fa)) continue;
        if (!first && !(w.ccd_state[h] == 0 && w.ccd_deps[h] == 0 && w.ccd_recompute[h] == 1)) continue;
        if (!ccd_target(w, h, o)) continue;
        if (!sweep_may_touch(w, h, o)) continue;
        Cast r = cast_one(w, h, o);
        if (r.hit) {
            // earliest time wins; equal times keep the lower handle (distance.rs:886-890)
            unsigned long long key = ((unsigned long long)__float_as_uint(r.t) << 32) | o;
            atomicMin(&w.ccd_best[h], key);
            if (w.ccd_hit) {
                uint32_t k = agg_inc(&w.ctr[C_CCD_HITS]);
                if (k < w.ccd_hit_cap) {
                    float4* rec = w.ccd_hit + (size_t)k * 3;
                    rec[0] = make_float4(r.t, __uint_as_float(o), __uint_as_float(h), __uint_as_float(tag));
                    rec[1] = st3(r.normal, 0.0f);
                    rec[2] = st3(r.point, 0.0f);
                }
            }
        }
    }
}
// Candidates with a fast body are listed once per substep (and the
// dependency counts taken); every cast round then walks that list, so the
// long cast loops fill whole warps instead of a few lanes of each.
__global__ void k_ccd_collect(DW w) {
    if (aborted(w)) return;
    if (w.ctr[C_FAST] == 0u) return;
    const uint32_t n = n_cand(w);
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        uint2 ab = w.cand[c];
        bool fa = w.fast[ab.x], fb = w.fast[ab.y];
        if (!fa && !fb) continue;
        w.fcand[agg_inc(&w.ctr[C_FCAND])] = c;
        if (fa && fb && ccd_target(w, ab.x, ab.y)) atomicAdd(&w.ccd_deps[ab.y], 1u);
    }
}
__global__ void k_ccd_cast(DW w, int first, uint32_t tag) {
    if (aborted(w)) return;
    if (w.ctr[C_FAST] == 0u || (!first && w.ctr[C_CCD_PENDING] == 0u)) return;
    const uint32_t n = w.ctr[C_FCAND];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        k_ccd_cast_one(w, first, w.fcand[i], tag);
}
// The record of each mover's winning cast of round `tag` (the one whose key
// equals the mover's best; keys are unique per mover).
__global__ void k_ccd_pick(DW w, uint32_t tag) {
    if (aborted(w) || !w.ccd_hit) return;
    if (w.ctr[C_FAST] == 0u || w.ctr[C_CCD_PENDING] == 0u) return;
    const uint32_t n = min(w.ctr[C_CCD_HITS], w.ccd_hit_cap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float4 r0 = w.ccd_hit[(size_t)k * 3];
        if (__float_as_uint(r0.w) != tag) continue;
        uint32_t o = __float_as_uint(r0.y), h = __float_as_uint(r0.z);
        unsigned long long key = ((unsigned long long)__float_as_uint(r0.x) << 32) | o;
        if (w.ccd_best[h] == key) w.ccd_win[h] = k;
    }
}

// recorded: the winner's record may be used (its cast saw the final poses)
static __device__ void ccd_apply(const DW& w, uint32_t h, bool recorded) {
    unsigned long long key = w.ccd_best[h];
    bool moved = false;
    if (key != ~0ull) {
        uint32_t o = (uint32_t)(key & 0xffffffffu);
        Cast r;
        const uint32_t k = recorded && w.ccd_win ? w.ccd_win[h] : ~0u;
        if (k != ~0u) {
            const float4* rec = w.ccd_hit + (size_t)k * 3;
            r = Cast{true, rec[0].x, ld3(rec[1]), ld3(rec[2])};
        } else {
            r = cast_one(w, h, o);  // the winning cast again: same inputs, same t and normal
        }
        V3 disp = ld3(w.vel[h]) * w.dt;
        float L = fmaxf(len(disp), MIN_TOI_DISP_LENGTH);
        float frac = fclamp(r.t / L, 0.0f, 1.0f);
        float e = fminf(w.mat[h].x, w.mat[o].x);
        if (w.ccd_ev_o) {
            // a swept impact is a hit event (mod.rs:946-960)
            float approach = -dot(ld3(w.pre_vel[h]) - ld3(w.pre_vel[o]), r.normal);
            if (approach > 1.0f) {
                w.ccd_ev_o[h] = (int32_t)o;
                w.ccd_ev_p[h] = st3(r.point, approach);
                w.ccd_ev_n[h] = st3(h < o ? -r.normal : r.normal, 0.0f);
            }
        }
        w.pos[h] = st3(ld3(w.pos[h]) + disp * frac, 0.0f);
        V3 v = ld3(w.vel[h]);
        float vn = dot(v, r.normal);
        float bounce = 0.0f;
        if (vn < 0.0f) {
            bounce = vn < -CCD_BOUNCE_SPEED ? 1.0f + e : 1.0f;
            w.vel[h] = st3(v - r.normal * (bounce * vn), 0.0f);
        }
        if (w.sort_static) {
            w.ccd_rec[2 * h] = st3(r.normal, bounce);
            w.ccd_rec[2 * h + 1] = make_float4(frac * w.dt, 1.0f, 0.0f, 0.0f);
        }
        wake_body(w, o);
        w.sleep_timer[h] = 0.0f;
        agg_inc(&w.ctr[C_CCD]);
        moved = true;
    }
    w.ccd_state[h] = moved ? 2 : 1;
}
__global__ void k_ccd_finalize(DW w, int round, int last) {
    if (aborted(w)) return;
    if (w.ctr[C_CCD_PENDING] == 0u) return;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.ctr[C_FAST]) return;
    uint32_t h = w.fbody[i];
    if (w.ccd_state[h] != 0) return;
    const bool waiting = w.ccd_deps[h] != 0;
    if (waiting) {
        if (!last) return;
        atomicAdd(&w.ctr[C_CCD_LEFT], 1u);  // dependency chain longer than the bounded rounds
    }
    ccd_apply(w, h, !waiting);
    w.ccd_recompute[h] = (uint8_t)(16 + round);  // "finalised in this round"
    atomicSub(&w.ctr[C_CCD_PENDING], 1u);
}
static __device__ __forceinline__ void k_ccd_release_one(const DW& w, int round, uint32_t c) {
    uint2 ab = w.cand[c];
    if (!w.fast[ab.x] || !w.fast[ab.y]) return;
    if (w.ccd_recompute[ab.x] != (uint8_t)(16 + round)) return;
    if (!ccd_target(w, ab.x, ab.y)) return;
    atomicSub(&w.ccd_deps[ab.y], 1u);
    if (w.ccd_state[ab.x] == 2) w.ccd_recompute[ab.y] = 1;  // the earlier mover moved: recast
}
__global__ void k_ccd_release(DW w, int round) {
    if (aborted(w)) return;
    if (w.ctr[C_CCD_PENDING] == 0u) return;
    const uint32_t n = w.ctr[C_FCAND];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        k_ccd_release_one(w, round, w.fcand[i]);
}

__global__ void k_ccd_reset(DW w) {
    if (aborted(w)) return;
    if (w.ctr[C_CCD_PENDING] == 0u) return;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.ctr[C_FAST]) return;
    uint32_t h = w.fbody[i];
    if (w.ccd_state[h] == 0 && w.ccd_deps[h] == 0 && w.ccd_recompute[h] == 1) {
        w.ccd_best[h] = ~0ull;
        if (w.ccd_win) w.ccd_win[h] = ~0u;
    }
}
__global__ void k_ccd_clear_recast(DW w) {
    if (aborted(w)) return;
    if (w.ctr[C_CCD_PENDING] == 0u) return;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.ctr[C_FAST]) return;
    uint32_t h = w.fbody[i];
    if (w.ccd_state[h] == 0 && w.ccd_deps[h] == 0 && w.ccd_recompute[h] == 1) w.ccd_recompute[h] = 0;
}
void launch_ccd(const DW& w, cudaStream_t st) {
    if (!w.enable_ccd) return;
    unsigned gb = nblk(w.N, 256);
    k_ccd_init<<<gb, 256, 0, st>>>(w);
    k_ccd_collect<<<gsz(w.cand_cap, 256), 256, 0, st>>>(w);
    const unsigned gh = w.ccd_hit ? gsz(w.ccd_hit_cap, 256) : 0u;
    k_ccd_cast<<<gsz(w.cand_cap, 128), 128, 0, st>>>(w, 1, 0u);
    if (gh) k_ccd_pick<<<gh, 256, 0, st>>>(w, 0u);
    for (int r = 0; r < CCD_ROUNDS; r++) {
        bool last = r == CCD_ROUNDS - 1;
        k_ccd_finalize<<<gb, 256, 0, st>>>(w, r, last ? 1 : 0);
        if (last) break;
        k_ccd_release<<<gsz(w.cand_cap, 256), 256, 0, st>>>(w, r);
        k_ccd_reset<<<gb, 256, 0, st>>>(w);
        k_ccd_cast<<<gsz(w.cand_cap, 128), 128, 0, st>>>(w, 0, (uint32_t)(r + 1));
        if (gh) k_ccd_pick<<<gh, 256, 0, st>>>(w, (uint32_t)(r + 1));
        k_ccd_clear_recast<<<gb, 256, 0, st>>>(w);
    }
}

}  // namespace avbd
