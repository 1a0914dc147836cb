/*
 * rt/camera.hpp — the reference's Camera (include/rt/camera.hpp:9-61):
 * position, normalised direction, and the right / up vectors scaled by the
 * vertical field of view and the aspect ratio (Camera::set,
 * src/rt/camera.cpp:31-59, computed by rt_camera_set).
 */
#pragma once
#ifndef RT_CAMERA_HPP
#define RT_CAMERA_HPP

#include "../rt_cuda.h"

struct vec3 {
    float s[3];
    vec3() : s{0.f, 0.f, 0.f} {}
    vec3(float x, float y, float z) : s{x, y, z} {}
    float& operator[](int i) { return s[i]; }
    float operator[](int i) const { return s[i]; }
};

inline vec3 makeVector(float x, float y, float z) { return vec3(x, y, z); }

class Camera {
public:
    vec3 pos;
    vec3 dir;
    vec3 right;
    vec3 up;
    bool right_handed;
    float fov;
    float aspect;

    Camera();
    Camera(const vec3& Position, const vec3& Direction, const vec3& Up, float FOV, float Aspect,
           bool RightHanded = false);
    void set(const vec3& Position, const vec3& Direction, const vec3& Up, float FOV = 0.f,
             float Aspect = 0.f, bool RightHanded = false);

    /* The four float4 vectors the primary-ray kernel takes. */
    rt_camera to_rt() const;
};

#endif /* RT_CAMERA_HPP */
