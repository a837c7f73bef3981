// avbd_static.cu — allocation-free stepping of one small scene.
//
// Some callers cannot call cudaMalloc: code running under an allocator it
// does not own (a host engine that hands out only its own pools, a process
// whose CUDA memory is capped or pre-reserved, a context where allocation
// would synchronise a stream that must not stall).  For them,
// avbd_scene_step_static steps one small scene through the same kernels as
// an AvbdWorld, with every device buffer carved out of one file-scope
// device array declared below.  Nothing is allocated: no cudaMalloc,
// cudaFree, stream or event creation, no pinned memory.
//
// Limits: at most AVBD_STATIC_MAX_BODIES (128) bodies, no joints, at most
// AVBD_STATIC_PAIR_CAP (2048) broadphase candidates (= contact pair slots)
// per substep.  The array is AVBD_STATIC_SCRATCH_BYTES (3.4 MB) and every GPU
// that loads this library holds it until the process exits.
//
// Every call shares the array.  A call starts from the bodies it is given
// (no warm contact state carries over from an earlier call: everything that
// must start at zero is cleared at the start of the call), so two calls that
// overlap on the GPU — from two host threads, or on two streams — race on
// the array and must not be issued.
//
// The first call on a device is where the CUDA runtime loads this library's
// device code (lazy module loading, the default): loading places the array
// and the kernels in device memory.  A caller that reserves or caps device
// memory must therefore make one call on each device before it does so (or
// run with CUDA_MODULE_LOADING=EAGER, which loads everything when the
// context is created); the calls after that allocate nothing.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "avbd_kernels.h"

using namespace avbd;

namespace {

constexpr uint32_t MAXB = AVBD_STATIC_MAX_BODIES;
constexpr uint32_t PCAP = AVBD_STATIC_PAIR_CAP;
constexpr size_t STATIC_BYTES = AVBD_STATIC_SCRATCH_BYTES;

}  // namespace

// The scratch of the allocation-free entry point.  In host code this name is
// only a host-side stand-in: its device address comes from
// cudaGetSymbolAddress (static_base() below).
static __device__ __align__(256) unsigned char g_scene_scratch[STATIC_BYTES];

namespace {

// The array's device address on the caller's current device.  It is looked
// up on every call (a table lookup once the module is loaded), so a context
// that was reset and re-created (cudaDeviceReset) gets the new address and
// never a stale one; the first lookup on a device loads the module.
int static_base(unsigned char** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scene_scratch) != cudaSuccess || !p) return AVBD_ERR_DEVICE;
    *out = (unsigned char*)p;
    return AVBD_OK;
}

struct Carver {
    unsigned char* base;
    size_t off = 0;
    bool ok = true;
    template <class T> T* take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        T* p = (T*)(base + off);
        off += (n ? n : 1) * sizeof(T);
        if (off > STATIC_BYTES) ok = false;
        return p;
    }
};

float bound_of(const AvbdBody& b) {  // rows.rs:253-292
    const float* p = b.shape_params;
    switch (b.shape) {
        case AVBD_SHAPE_SPHERE: return p[0];
        case AVBD_SHAPE_BOX: return std::sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]);
        case AVBD_SHAPE_CAPSULE: return p[1] + p[0];
        case AVBD_SHAPE_CYLINDER:
        case AVBD_SHAPE_CONE: return std::sqrt(p[0] * p[0] + p[1] * p[1]);
        default: return INFINITY;
    }
}
void inertia_of(const AvbdBody& b, float m, float out[3]) {  // collision/shape.rs:713-790
    const float* sp = b.shape_params;
    out[0] = out[1] = out[2] = 0.0f;
    if (!(m > 0.0f) || !std::isfinite(m)) return;
    if (b.shape == AVBD_SHAPE_SPHERE) {
        out[0] = out[1] = out[2] = 0.4f * m * sp[0] * sp[0];
    } else if (b.shape == AVBD_SHAPE_BOX) {
        float sx = sp[0] * 2.0f, sy = sp[1] * 2.0f, sz = sp[2] * 2.0f;
        float x = sx * sx, y = sy * sy, z = sz * sz, k = m / 12.0f;
        out[0] = k * (y + z);
        out[1] = k * (z + x);
        out[2] = k * (x + y);
    } else if (b.shape == AVBD_SHAPE_CAPSULE) {
        float r = sp[0], h = sp[1];
        float ixz = 0.25f * m * (r * r) + (m / 3.0f) * h * r + 0.25f * m * h * h;
        out[0] = ixz;
        out[1] = 0.5f * m * r * r;
        out[2] = ixz;
    } else if (b.shape == AVBD_SHAPE_CYLINDER || b.shape == AVBD_SHAPE_CONE) {
        float r = sp[0], h = sp[1];
        bool cyl = b.shape == AVBD_SHAPE_CYLINDER;
        float ixz = m * (3.0f * r * r + (cyl ? 4.0f : 8.0f) * h * h) / (cyl ? 12.0f : 20.0f);
        out[0] = ixz;
        out[1] = (cyl ? 0.5f : 0.3f) * m * r * r;
        out[2] = ixz;
    }
}

__global__ void k_static_in(DW w, const AvbdBody* in, uint32_t n) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= n) return;
    const AvbdBody& b = in[h];
    w.pos[h] = make_float4(b.position[0], b.position[1], b.position[2], 0.0f);
    w.rot[h] = make_float4(b.orientation[0], b.orientation[1], b.orientation[2], b.orientation[3]);
    w.prev_pos[h] = w.pos[h];
    w.prev_rot[h] = w.rot[h];
    w.vel[h] = make_float4(b.velocity[0], b.velocity[1], b.velocity[2], 0.0f);
    w.angvel[h] = make_float4(b.angular_velocity[0], b.angular_velocity[1], b.angular_velocity[2], 0.0f);
    w.torque[h] = make_float4(b.torque[0], b.torque[1], b.torque[2], 0.0f);
    w.mass[h] = b.mass;
    w.inv_mass[h] = b.inv_mass;
    w.inertia[h] = make_float4(b.inertia[0], b.inertia[1], b.inertia[2], 0.0f);
    w.mat[h] = make_float4(b.restitution, b.friction, b.rolling_friction, b.torsion_friction);
    w.friction_t[h] = b.friction_transverse;
    w.filter[h] = make_uint2(b.collision_layer, b.collision_mask);
    w.comp[h] = -1;  // no joints
}
__global__ void k_static_out(DW w, AvbdBody* io, uint32_t n) {  // io holds the caller's records
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= n) return;
    AvbdBody& b = io[h];
    float4 p = w.pos[h], q = w.rot[h], v = w.vel[h], om = w.angvel[h], tq = w.torque[h], in = w.inertia[h];
    b.position[0] = p.x; b.position[1] = p.y; b.position[2] = p.z;
    b.orientation[0] = q.x; b.orientation[1] = q.y; b.orientation[2] = q.z; b.orientation[3] = q.w;
    b.velocity[0] = v.x; b.velocity[1] = v.y; b.velocity[2] = v.z;
    b.angular_velocity[0] = om.x; b.angular_velocity[1] = om.y; b.angular_velocity[2] = om.z;
    b.torque[0] = tq.x; b.torque[1] = tq.y; b.torque[2] = tq.z;
    b.mass = w.mass[h];
    b.inv_mass = w.inv_mass[h];
    b.inertia[0] = in.x; b.inertia[1] = in.y; b.inertia[2] = in.z;
}

}  // namespace

extern "C" int avbd_scene_step_static(const AvbdParams* params, const AvbdBody* bodies, uint32_t n,
                                      int32_t substeps, AvbdBody* out) {
    if (!params || !bodies || !out || n == 0 || substeps < 0) return AVBD_ERR_INVALID_ARG;
    if (n > MAXB) return AVBD_ERR_CAPACITY;
    if (!(params->step_dt > 0.0f) || !std::isfinite(params->step_dt) || params->iterations < 0)
        return AVBD_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; i++) {
        const float* f = bodies[i].position;
        for (int k = 0; k < 16; k++)
            if (!std::isfinite(f[k])) return AVBD_ERR_NONFINITE;
        if (!std::isfinite(bodies[i].mass) || !std::isfinite(bodies[i].inv_mass)) return AVBD_ERR_NONFINITE;
        // hull, rounded and compound tables live in worlds
        if (bodies[i].shape >= AVBD_SHAPE_HULL) return AVBD_ERR_UNSUPPORTED;
    }
    unsigned char* base = nullptr;
    int rc = static_base(&base);
    if (rc) return rc;
    const uint32_t N = n, S = 1;
    cudaStream_t st = cudaStreamPerThread;
    Carver cv{base};
    DW w{};
    w.N = (int)N;
    w.S = (int)S;
    w.J = 0;
    w.dt = params->step_dt;
    w.gravity = V3{params->gravity[0], params->gravity[1], params->gravity[2]};
    w.iterations = params->iterations;
    w.enable_sleep = params->enable_sleep;
    w.enable_ccd = params->enable_ccd;
    w.cand_cap = PCAP;
    w.pair_cap = PCAP;
    w.max_cols = MAX_COLOURS;
    uint32_t* scene_off = cv.take<uint32_t>(S + 1);
    uint32_t* scene_of = cv.take<uint32_t>(N);
    uint32_t* plane_off = cv.take<uint32_t>(S + 1);
    uint32_t* plane_list = cv.take<uint32_t>(N);
    w.scene_off = scene_off;
    w.scene_of = scene_of;
    w.plane_off = plane_off;
    w.plane_list = plane_list;
    float4** f4[] = {&w.pos, &w.rot, &w.vel, &w.angvel, &w.torque, &w.pos0, &w.rot0, &w.inertial, &w.inertial_rot,
                     &w.prev_pos, &w.prev_rot, &w.inertia, &w.inertia_rest, &w.mat, &w.shp,
                     &w.aabb_lo, &w.aabb_hi};
    for (float4** p : f4) *p = cv.take<float4>(N);
    float** f1[] = {&w.inv_mass, &w.inv_mass_rest, &w.mass, &w.friction_t, &w.sleep_timer};
    for (float** p : f1) *p = cv.take<float>(N);
    w.info = cv.take<uint32_t>(N);
    w.asleep = cv.take<uint32_t>(N);
    w.filter = cv.take<uint2>(N);
    w.colour = cv.take<int32_t>(N);
    w.comp = cv.take<int32_t>(N);
    w.j_kind = cv.take<uint32_t>(1);
    w.j_ab = cv.take<uint2>(1);
    float4** jf[] = {&w.j_la, &w.j_lb, &w.j_axa, &w.j_axb, &w.j_lim, &w.j_lam_l, &w.j_lam_a, &w.j_pen_l, &w.j_pen_a};
    for (float4** p : jf) *p = cv.take<float4>(1);
    w.jofs = cv.take<uint32_t>(N + 1);
    w.jlist = cv.take<uint32_t>(1);
    struct Buf {
        uint2* ab;
        float4* nn;
        float2* mu;
        uint32_t* np;
        float4 *ra, *rb, *lam, *pen, *roll;
        int32_t* matched;
        uint32_t* offA;
    } pb[2];
    for (auto& b : pb) {
        b.ab = cv.take<uint2>(PCAP);
        b.nn = cv.take<float4>(PCAP);
        b.mu = cv.take<float2>(PCAP);
        b.np = cv.take<uint32_t>(PCAP);
        b.ra = cv.take<float4>((size_t)PCAP * MAX_PTS);
        b.rb = cv.take<float4>((size_t)PCAP * MAX_PTS);
        b.lam = cv.take<float4>((size_t)PCAP * MAX_PTS);
        b.pen = cv.take<float4>((size_t)PCAP * MAX_PTS);
        b.roll = cv.take<float4>((size_t)PCAP * MAX_PTS);
        b.matched = cv.take<int32_t>((size_t)PCAP * MAX_PTS);
        b.offA = cv.take<uint32_t>(N + 1);
    }
    w.offB = cv.take<uint32_t>(N + 1);
    w.listB = cv.take<uint32_t>(PCAP);
    w.cand = cv.take<uint2>(PCAP);
    w.keep = cv.take<uint8_t>(PCAP);
    w.cnt = cv.take<uint32_t>(N + 1);
    w.cur = cv.take<uint32_t>(N + 1);
    w.slot_c = cv.take<uint32_t>(PCAP);
    w.boxlist = cv.take<uint32_t>(PCAP);
    w.clist = cv.take<uint32_t>(PCAP);
    w.bd_pa = cv.take<float4>(PCAP);
    w.bd_pb = cv.take<float4>(PCAP);
    w.sort_key = cv.take<uint32_t>(1);
    w.sort_idx = cv.take<uint32_t>(1);
    w.kin = cv.take<float4>((size_t)N * 4);
    w.fbody = cv.take<uint32_t>(N);
    w.fcand = cv.take<uint32_t>(PCAP);
    w.fast = cv.take<uint8_t>(N);
    w.ccd_best = cv.take<unsigned long long>(N);
    w.ccd_deps = cv.take<uint32_t>(N);
    w.ccd_state = cv.take<uint8_t>(N);
    w.ccd_recompute = cv.take<uint8_t>(N);
    w.flag = cv.take<uint8_t>(N);
    w.comp_flag = cv.take<uint32_t>(N);
    w.col_cnt = cv.take<uint32_t>(2 * MAX_COLOURS + 2);
    w.col_list = cv.take<uint32_t>(N);
    w.col_key = cv.take<uint32_t>(N);
    w.col_key2 = cv.take<uint32_t>(N);
    w.col_val = cv.take<uint32_t>(N);
    w.col_hist = cv.take<uint32_t>(radix_hist_words(N));
    w.ctr = cv.take<uint32_t>(C_NUM);
    uint32_t* small = cv.take<uint32_t>(1);
    uint32_t* scan_tmp = cv.take<uint32_t>(scan_tmp_words(radix_hist_words(N) + N + 1) + 16);
    AvbdBody* stage = cv.take<AvbdBody>(N);
    if (!cv.ok) return AVBD_ERR_CAPACITY;

    // clear the whole region this call uses: counters, previous-generation
    // pair offsets and B-side lists (no pairs yet), sleep state
    if (cudaMemsetAsync(base, 0, cv.off, st) != cudaSuccess) return AVBD_ERR_DEVICE;
    // host-derived per-body data (same rules as a world's upload)
    uint32_t h_scene_off[2] = {0, N}, h_plane_off[2] = {0, 0}, h_plane_list[MAXB], h_scene_of[MAXB], h_info[MAXB];
    float4 h_shp[MAXB], h_inrest[MAXB];
    float h_invrest[MAXB];
    for (uint32_t h = 0; h < N; h++) {
        const AvbdBody& b = bodies[h];
        h_scene_of[h] = 0;
        if (b.shape == AVBD_SHAPE_HALFSPACE) h_plane_list[h_plane_off[1]++] = h;
        h_info[h] = (b.shape & 15u) | ((b.body_type & 3u) << 4) | ((b.flags & AVBD_FLAG_TRIGGER) ? 64u : 0u);
        h_shp[h] = make_float4(b.shape_params[0], b.shape_params[1], b.shape_params[2], bound_of(b));
        bool free_mass = b.mass > 0.0f && std::isfinite(b.mass);
        float in[3];
        inertia_of(b, free_mass ? b.mass : 0.0f, in);
        h_inrest[h] = make_float4(in[0], in[1], in[2], 0.0f);
        h_invrest[h] = free_mass ? 1.0f / b.mass : 0.0f;
    }
    uint32_t zero = 0;
    struct Up {
        void* dst;
        const void* src;
        size_t bytes;
    } ups[] = {
        {scene_off, h_scene_off, 8}, {plane_off, h_plane_off, 8}, {plane_list, h_plane_list, 4 * N},
        {scene_of, h_scene_of, 4 * N}, {w.info, h_info, 4 * N}, {w.shp, h_shp, 16 * N},
        {w.inertia_rest, h_inrest, 16 * N}, {w.inv_mass_rest, h_invrest, 4 * N}, {small, &zero, 4},
        {stage, bodies, sizeof(AvbdBody) * N},
    };
    for (const Up& u : ups)
        if (u.bytes && cudaMemcpyAsync(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
            return AVBD_ERR_DEVICE;
    k_static_in<<<1, MAXB, 0, st>>>(w, stage, N);
    BroadphasePlan plan;
    plan.small_scenes = small;
    plan.n_small = 1;
    plan.scan_tmp = scan_tmp;
    Tune tune;  // exact build, one thread per body: the defaults of a world
    int cur = 0;
    uint32_t ctr[C_NUM];
    bool colour_overflow = false;  // a world reports it the same way, after finishing the substep
    for (int s = 0; s < substeps && !colour_overflow; s++) {
        cur = 1 - cur;  // the previous generation becomes `old`
        const Buf& c = pb[cur];
        const Buf& o = pb[1 - cur];
        w.p_ab = c.ab; w.p_n = c.nn; w.p_mu = c.mu; w.p_np = c.np;
        w.q_ra = c.ra; w.q_rb = c.rb; w.q_lam = c.lam; w.q_pen = c.pen; w.q_roll = c.roll; w.q_matched = c.matched;
        w.offA = c.offA;
        w.o_ab = o.ab; w.o_n = o.nn; w.o_np = o.np;
        w.oq_ra = o.ra; w.oq_rb = o.rb; w.oq_lam = o.lam; w.oq_pen = o.pen; w.oq_roll = o.roll;
        w.o_offA = o.offA;
        launch_begin_substep(w, st);
        launch_wake_joint_motion(w, st);
        launch_torque(w, st);
        launch_broadphase(w, plan, st);
        launch_ccd(w, st);
        launch_discovery(w, scan_tmp, st);
        launch_post_discovery(w, scan_tmp, st);
        launch_colouring(w, tune, scan_tmp, st);
        if (cudaMemcpyAsync(ctr, w.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return AVBD_ERR_DEVICE;
        if (ctr[C_ERR] & E_CAND_OVERFLOW) return AVBD_ERR_CAPACITY;  // more than PCAP candidates
        if (ctr[C_ERR] & E_COLOUR_OVERFLOW) colour_overflow = true;
        int ncol = (int)ctr[C_NCOL];
        for (int it = 0; it < w.iterations; it++) launch_iteration(w, tune, ncol, st);
        launch_finish_substep(w, tune, st);
    }
    if (colour_overflow) {
        // more colours than a launch covers: out is left untouched
        return cudaStreamSynchronize(st) == cudaSuccess ? AVBD_ERR_CAPACITY : AVBD_ERR_DEVICE;
    }
    k_static_out<<<1, MAXB, 0, st>>>(w, stage, N);
    if (cudaGetLastError() != cudaSuccess) return AVBD_ERR_DEVICE;
    if (cudaMemcpyAsync(out, stage, sizeof(AvbdBody) * N, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return AVBD_ERR_DEVICE;
    return AVBD_OK;
}
