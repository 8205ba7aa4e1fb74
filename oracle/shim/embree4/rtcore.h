/*
 * Minimal stand-in for Embree 4's rtcore.h, written for this project.
 *
 * TEST INFRASTRUCTURE: lets the unmodified reference source
 * (mo_lradtopo_horayzon.cpp, which includes <embree4/rtcore.h> at line 13)
 * compile here, where Embree is not installed. It declares only the names the
 * reference uses (cpp:370-459); their meaning follows Embree 4's public API
 * documentation. The geometry query behind rtcOccluded1 is the project's own
 * (hz_occlusion.h), not Embree's, so results pin the reference's code around
 * the query, not Embree's arithmetic.
 */
#ifndef HZ_SHIM_EMBREE4_RTCORE_H
#define HZ_SHIM_EMBREE4_RTCORE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct RTCDeviceTy* RTCDevice;
typedef struct RTCSceneTy* RTCScene;
typedef struct RTCGeometryTy* RTCGeometry;

enum RTCError {
    RTC_ERROR_NONE = 0,
    RTC_ERROR_UNKNOWN = 1,
    RTC_ERROR_INVALID_ARGUMENT = 2,
    RTC_ERROR_INVALID_OPERATION = 3,
    RTC_ERROR_OUT_OF_MEMORY = 4
};
enum RTCSceneFlags { RTC_SCENE_FLAG_NONE = 0, RTC_SCENE_FLAG_ROBUST = (1 << 2) };
enum RTCGeometryType { RTC_GEOMETRY_TYPE_TRIANGLE = 0 };
enum RTCBufferType { RTC_BUFFER_TYPE_INDEX = 0, RTC_BUFFER_TYPE_VERTEX = 1 };
enum RTCFormat { RTC_FORMAT_UNDEFINED = 0, RTC_FORMAT_UINT3 = 0x5003, RTC_FORMAT_FLOAT3 = 0x9003 };

typedef void (*RTCErrorFunction)(void* userPtr, enum RTCError code, const char* str);

struct RTCRay {
    float org_x, org_y, org_z;
    float tnear;
    float dir_x, dir_y, dir_z;
    float time;
    float tfar;
    unsigned int mask;
    unsigned int id;
    unsigned int flags;
};

struct RTCOccludedArguments;

RTCDevice rtcNewDevice(const char* config);
enum RTCError rtcGetDeviceError(RTCDevice device);
void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction fn, void* userPtr);
RTCScene rtcNewScene(RTCDevice device);
void rtcSetSceneFlags(RTCScene scene, enum RTCSceneFlags flags);
RTCGeometry rtcNewGeometry(RTCDevice device, enum RTCGeometryType type);
void* rtcSetNewGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type,
                              unsigned int slot, enum RTCFormat format,
                              size_t byteStride, size_t itemCount);
void rtcSetSharedGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type,
                                unsigned int slot, enum RTCFormat format,
                                const void* ptr, size_t byteOffset,
                                size_t byteStride, size_t itemCount);
void rtcCommitGeometry(RTCGeometry geometry);
unsigned int rtcAttachGeometry(RTCScene scene, RTCGeometry geometry);
void rtcReleaseGeometry(RTCGeometry geometry);
void rtcCommitScene(RTCScene scene);
#ifdef __cplusplus
void rtcOccluded1(RTCScene scene, struct RTCRay* ray,
                  struct RTCOccludedArguments* args = NULL);
#else
void rtcOccluded1(RTCScene scene, struct RTCRay* ray,
                  struct RTCOccludedArguments* args);
#endif

#ifdef __cplusplus
}
#endif
#endif
