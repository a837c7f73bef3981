// The device's row stamp and 6x6 LDL^T (ornis_gb300/csrc/avbd_rows.cuh) run
// on the GPU on the reference's known-answer systems
// (crates/physics/tests/gpu_batches.rs:781-856 stamp, :863-898 solve and
// breakdown).  Prints the results as text for tests/test_gpu_rows_kat.py.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../ornis_gb300/csrc/avbd_rows.cuh"

using namespace avbd;

struct Out {
    float stamp_h[2][21], stamp_r[2][6];  // side +1, side -1
    int ok[3];                              // SPD, zero, negative pivot
    float x[3][6];
};

__global__ void k_kat(Out* o) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int side = 0; side < 2; side++) {
        Sys s;
        for (int k = 0; k < 21; k++) s.h[k] = 0.0f;
        for (int k = 0; k < 6; k++) s.r[k] = 0.0f;
        stamp_row(s, V3{0.0f, 1.0f, 0.0f}, 2.0f, 3.0f, V3{1.0f, 0.0f, 0.0f}, side ? -1.0f : 1.0f);
        for (int k = 0; k < 21; k++) o->stamp_h[side][k] = s.h[k];
        for (int k = 0; k < 6; k++) o->stamp_r[side][k] = s.r[k];
    }
    const float rhs[6] = {1.0f, -2.0f, 3.0f, -4.0f, 5.0f, -6.0f};
    for (int c = 0; c < 3; c++) {
        Sys s;
        for (int i = 0; i < 6; i++)
            for (int j = 0; j <= i; j++) {
                float v = i == j ? 4.0f + (float)i : 0.1f * ((float)(i + j) + 1.0f);
                if (c == 1) v = 0.0f;
                if (c == 2 && i == 0 && j == 0) v = -1.0f;
                s.h[tri(i, j)] = v;
            }
        for (int i = 0; i < 6; i++) s.r[i] = -rhs[i];  // the solve returns x with H x = -r
        float x[6] = {0, 0, 0, 0, 0, 0};
        o->ok[c] = solve_6x6(s, x) ? 1 : 0;
        for (int i = 0; i < 6; i++) o->x[c][i] = x[i];
    }
}

int main() {
    Out* d = nullptr;
    if (cudaMalloc(&d, sizeof(Out)) != cudaSuccess) return 2;
    k_kat<<<1, 32>>>(d);
    Out h;
    if (cudaMemcpy(&h, d, sizeof(Out), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
    for (int side = 0; side < 2; side++) {
        printf("stamp%d", side);
        for (int k = 0; k < 21; k++) printf(" %a", h.stamp_h[side][k]);
        for (int k = 0; k < 6; k++) printf(" %a", h.stamp_r[side][k]);
        printf("\n");
    }
    for (int c = 0; c < 3; c++) {
        printf("solve%d %d", c, h.ok[c]);
        for (int i = 0; i < 6; i++) printf(" %a", h.x[c][i]);
        printf("\n");
    }
    cudaFree(d);
    return 0;
}
