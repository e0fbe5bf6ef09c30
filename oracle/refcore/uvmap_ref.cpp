// uvmap_ref.cpp -- texture-space face map of the normal-map mode computed
// with the reference's own host ray/triangle test.  Test infrastructure
// only: it checks the oracle's restatement (orc_uv_face_map) and makes the
// golden face-map fixtures; the product never loads it.
//
// rayTriangleIntersectHost is compiled from the reference source
// (cpp/src/Renderer/CUDABasedRasterization.cpp:158-236) and linked in
// unchanged; this file drives it over the texel boxes exactly as the
// reference's first-call loop does (:252-294), serially in face order.
#include <cmath>
#include <vector_types.h>

bool rayTriangleIntersectHost(float3 orig, float3 dir, float3 v0, float3 v1, float3 v2, float &t, float &a, float &b);

static float3 f3(float x, float y, float z) {
    float3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}

extern "C" {

// The reference object file also references the GPU launcher of its
// renderBuffers(); nothing here calls it.
void renderBuffersGPU(void *) {}

// owner [Ht*Wt] = face or -1; abc [Ht*Wt*3] = (a, b, c) or 0.
void refuv_face_map(const float *uvs, int F, int Ht, int Wt, int *owner, float *abc) {
    for (long i = 0; i < (long)Ht * Wt; ++i) {
        owner[i] = -1;
        abc[3 * i] = abc[3 * i + 1] = abc[3 * i + 2] = 0.0f;
    }
    for (int f = 0; f < F; ++f) {
        const float *c = uvs + 6 * (long)f;
        float3 t0 = f3(Wt * c[0], Ht * (1.f - c[1]), 0.f);
        float3 t1 = f3(Wt * c[2], Ht * (1.f - c[3]), 0.f);
        float3 t2 = f3(Wt * c[4], Ht * (1.f - c[5]), 0.f);
        int xMin = std::fmax(std::fmin(t0.x, std::fmin(t1.x, t2.x)) - 2, 0);
        int xMax = std::fmin(std::fmax(t0.x, std::fmax(t1.x, t2.x)) + 2, Wt);
        int yMin = std::fmax(std::fmin(t0.y, std::fmin(t1.y, t2.y)) - 2, 0);
        int yMax = std::fmin(std::fmax(t0.y, std::fmax(t1.y, t2.y)) + 2, Ht);
        for (int x = xMin; x < xMax; x++)
            for (int y = yMin; y < yMax; y++) {
                float a, b, cc, t;
                bool hit = rayTriangleIntersectHost(f3(x + 0.5f, y + 0.5f, 1.f), f3(0.f, 0.f, -1.f), t0, t1, t2, t, a, b);
                if (!hit)
                    a = b = cc = -1.f;
                else
                    cc = 1.f - a - b;
                if (a != -1.f && b != -1.f && cc != -1.f) {
                    long i = (long)y * Wt + x;
                    owner[i] = f;
                    abc[3 * i] = a;
                    abc[3 * i + 1] = b;
                    abc[3 * i + 2] = cc;
                }
            }
    }
}

}  // extern "C"
