/* A C caller of libornis_avbd.so through include/ornis_avbd.h: the call
 * sequence a host engine's dispatch makes (the Rust GpuAvbdDispatch of
 * rust/ornis-avbd-gb300 does the same).
 *
 *   seam cpu  — no device: ABI version, default parameters, body records of
 *               every primitive shape (avbd_body_init)
 *   seam gpu  — a world on device 0: bodies and a ball joint added, then per
 *               step the host records written back, the accumulator step,
 *               the records read back and the contact events drained; at
 *               step 45 remove_joint and wake_body.  Prints the final poses.
 * Floats are printed in C99 hex so that a comparison can be bit for bit. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ornis_avbd.h"

#define CK(x)                                                        \
    do {                                                             \
        int rc_ = (x);                                               \
        if (rc_ != AVBD_OK) {                                        \
            fprintf(stderr, "%s failed: %d\n", #x, rc_);             \
            exit(1);                                                 \
        }                                                            \
    } while (0)

static void print_body(const AvbdBody* b) {
    printf("body %u %u", b->shape, b->body_type);
    for (int k = 0; k < 3; k++) printf(" %a", b->position[k]);
    for (int k = 0; k < 4; k++) printf(" %a", b->orientation[k]);
    printf(" %a %a", b->mass, b->inv_mass);
    for (int k = 0; k < 3; k++) printf(" %a", b->inertia[k]);
    printf(" %a %a\n", b->friction, b->restitution);
}

static int scene(AvbdBody* b) {
    const float floor_p[3] = {10, 1, 10}, floor_x[3] = {0, -1, 0};
    const float cube[3] = {0.5f, 0.5f, 0.5f}, ball[3] = {0.5f, 0, 0}, small[3] = {0.3f, 0.3f, 0.3f};
    int n = 0;
    CK(avbd_body_init(&b[n++], AVBD_SHAPE_BOX, floor_p, floor_x, 0.0f));
    for (int i = 0; i < 4; i++) {
        float x[3] = {0, 0.5f + 1.02f * (float)i, 0};
        CK(avbd_body_init(&b[n++], AVBD_SHAPE_BOX, cube, x, 1.0f));
    }
    const float bx[3] = {2.5f, 3, 0}, ax[3] = {-3, 4, 0}, px[3] = {-2, 4, 0};
    CK(avbd_body_init(&b[n++], AVBD_SHAPE_SPHERE, ball, bx, 1.0f));
    CK(avbd_body_init(&b[n++], AVBD_SHAPE_BOX, small, ax, 0.0f));
    CK(avbd_body_init(&b[n++], AVBD_SHAPE_BOX, small, px, 1.0f));
    return n;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    if (!strcmp(argv[1], "cpu")) {
        AvbdParams p;
        CK(avbd_default_params(&p));
        printf("abi %d\n", avbd_abi_version());
        printf("params %a %a %a %a %d %d %d %d\n", p.gravity[0], p.gravity[1], p.gravity[2], p.step_dt, p.iterations,
               p.max_substeps, p.enable_sleep, p.enable_ccd);
        const float sp[3] = {0.4f, 0, 0}, bx[3] = {0.5f, 0.25f, 1.0f}, cap[3] = {0.3f, 0.6f, 0};
        const float hs[3] = {0, 1, 0}, x[3] = {1, 2, 3};
        AvbdBody b;
        CK(avbd_body_init(&b, AVBD_SHAPE_SPHERE, sp, x, 2.0f));
        print_body(&b);
        CK(avbd_body_init(&b, AVBD_SHAPE_BOX, bx, x, 3.0f));
        print_body(&b);
        CK(avbd_body_init(&b, AVBD_SHAPE_CAPSULE, cap, x, 1.5f));
        print_body(&b);
        CK(avbd_body_init(&b, AVBD_SHAPE_HALFSPACE, hs, x, 0.0f));
        print_body(&b);
        return 0;
    }
    AvbdParams p;
    CK(avbd_default_params(&p));
    AvbdWorld* w = NULL;
    CK(avbd_world_create(&p, 0, &w));
    AvbdBody host[16];
    int n = scene(host);
    uint32_t first = 0;
    CK(avbd_world_add_bodies(w, host, (uint32_t)n, &first));
    AvbdJointDesc j;
    memset(&j, 0, sizeof(j));
    j.kind = AVBD_JOINT_BALL;
    j.body_a = 6;
    j.body_b = 7;
    j.local_anchor_a[0] = 0.5f;
    j.local_anchor_b[0] = -0.5f;
    uint32_t jh = 0;
    CK(avbd_world_add_joint(w, &j, &jh));
    AvbdContactEvent ev[256];
    uint32_t nev_total = 0;
    for (int s = 0; s < 90; s++) {
        CK(avbd_world_set_bodies(w, 0, (uint32_t)n, host));
        CK(avbd_world_step(w, 1.0f / 60.0f));
        CK(avbd_world_get_bodies(w, 0, (uint32_t)n, host));
        uint32_t nev = 0;
        CK(avbd_world_drain_contact_events(w, ev, 256, &nev));
        nev_total += nev;
        if (s == 45) {
            CK(avbd_world_remove_joint(w, jh));
            CK(avbd_world_wake_body(w, 2));
            CK(avbd_world_get_bodies(w, 0, (uint32_t)n, host));
        }
    }
    AvbdCounters c;
    CK(avbd_world_get_counters(w, &c));
    printf("events %u steps %llu\n", nev_total, (unsigned long long)c.steps);
    for (int i = 0; i < n; i++) print_body(&host[i]);
    CK(avbd_world_destroy(w));
    return 0;
}
