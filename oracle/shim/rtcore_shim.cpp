/*
 * rtcore_shim.cpp -- the project's implementation of the Embree 4 calls that
 * mo_lradtopo_horayzon.cpp makes (cpp:370-459), on top of hz_occlusion.h.
 *
 * TEST INFRASTRUCTURE: linked only into oracle/_ref (the unmodified reference
 * compiled here as a parity pin and CPU baseline). rtcCommitScene builds the
 * oracle's FP32 LBVH; rtcOccluded1 runs its watertight any-hit query and, on
 * a hit, sets ray->tfar = -inf as Embree does (the reference tests tfar < 0,
 * cpp:459).
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "embree4/rtcore.h"

#include "../hz_occlusion.h"
#define HZO_REAL float
#define HZO_SFX 32
#include "../hz_occlusion.h"
#undef HZO_REAL
#undef HZO_SFX

struct RTCDeviceTy {
    RTCErrorFunction fn = nullptr;
    void* user = nullptr;
};

struct RTCGeometryTy {
    std::vector<float> vertices;      /* owned (rtcSetNewGeometryBuffer) */
    const int* indices = nullptr;     /* shared (rtcSetSharedGeometryBuffer) */
    size_t n_vertices = 0, n_triangles = 0;
    size_t index_stride = 12;
};

struct RTCSceneTy {
    RTCDeviceTy* device = nullptr;
    std::vector<RTCGeometryTy*> geoms;
    hzo_bvh_32 bvh;
    bool built = false;
    RTCSceneTy() { std::memset(&bvh, 0, sizeof(bvh)); bvh.root = INT32_MIN; }
};

extern "C" {

RTCDevice rtcNewDevice(const char*) { return new RTCDeviceTy(); }

enum RTCError rtcGetDeviceError(RTCDevice) { return RTC_ERROR_NONE; }

void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction fn, void* user) {
    if (device) { device->fn = fn; device->user = user; }
}

RTCScene rtcNewScene(RTCDevice device) {
    RTCSceneTy* s = new RTCSceneTy();
    s->device = device;
    return s;
}

void rtcSetSceneFlags(RTCScene, enum RTCSceneFlags) {}

RTCGeometry rtcNewGeometry(RTCDevice, enum RTCGeometryType) { return new RTCGeometryTy(); }

void* rtcSetNewGeometryBuffer(RTCGeometry g, enum RTCBufferType type, unsigned int,
                              enum RTCFormat, size_t byteStride, size_t itemCount) {
    if (type != RTC_BUFFER_TYPE_VERTEX || byteStride != 3 * sizeof(float)) return nullptr;
    g->vertices.assign(3 * itemCount, 0.0f);
    g->n_vertices = itemCount;
    return g->vertices.data();
}

void rtcSetSharedGeometryBuffer(RTCGeometry g, enum RTCBufferType type, unsigned int,
                                enum RTCFormat, const void* ptr, size_t byteOffset,
                                size_t byteStride, size_t itemCount) {
    if (type != RTC_BUFFER_TYPE_INDEX) return;
    g->indices = (const int*)((const char*)ptr + byteOffset);
    g->index_stride = byteStride;
    g->n_triangles = itemCount;
}

void rtcCommitGeometry(RTCGeometry) {}

unsigned int rtcAttachGeometry(RTCScene s, RTCGeometry g) {
    s->geoms.push_back(g);
    return (unsigned int)(s->geoms.size() - 1);
}

void rtcReleaseGeometry(RTCGeometry) {
    /* The scene keeps using the geometry; the reference never releases the
     * scene (cpp:647-649), so nothing is freed here. */
}

void rtcCommitScene(RTCScene s) {
    if (s->geoms.size() != 1) {
        if (s->device && s->device->fn)
            s->device->fn(s->device->user, RTC_ERROR_INVALID_OPERATION,
                          "shim supports exactly one triangle geometry");
        return;
    }
    RTCGeometryTy* g = s->geoms[0];
    std::vector<int> vot(3 * g->n_triangles);
    for (size_t t = 0; t < g->n_triangles; t++)
        for (int k = 0; k < 3; k++)
            vot[3 * t + k] = *(const int*)((const char*)g->indices + t * g->index_stride
                                           + k * sizeof(int));
    if (hzo_bvh_build_32(&s->bvh, g->vertices.data(), vot.data(),
                         (int)g->n_triangles) != 0) {
        if (s->device && s->device->fn)
            s->device->fn(s->device->user, RTC_ERROR_OUT_OF_MEMORY, "BVH build failed");
        return;
    }
    s->built = true;
}

void rtcOccluded1(RTCScene s, struct RTCRay* ray, struct RTCOccludedArguments*) {
    float o[3] = {ray->org_x, ray->org_y, ray->org_z};
    float d[3] = {ray->dir_x, ray->dir_y, ray->dir_z};
    hzo_ray_32 r;
    hzo_ray_setup_32(&r, o, d, ray->tnear, ray->tfar);
    hzo_counts c = {0, 0, 0};
    if (s->built && hzo_occluded_32(&s->bvh, &r, &c)) ray->tfar = -INFINITY;
}

}  // extern "C"
