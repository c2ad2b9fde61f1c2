// TEST INFRASTRUCTURE: a stand-in for the reference's camera.h (TCamera after TCamera::Set) over
// this library's sppm_camera_look_at.
#pragma once

#include "mesh.h"

class TCamera {
public:
    TVector3 origin, u, v, w;
    float distance = 0.0f;
    int width = 0, height = 0;

    void Set(TVector3 o, TVector3 lookat, int w_, int h_, float fov) {
        sppm_camera c;
        const float org[3] = {o.x, o.y, o.z}, at[3] = {lookat.x, lookat.y, lookat.z};
        sppm_camera_look_at(&c, org, at, (uint32_t)w_, (uint32_t)h_, fov);
        origin = TVector3(c.origin[0], c.origin[1], c.origin[2]);
        u = TVector3(c.u[0], c.u[1], c.u[2]);
        v = TVector3(c.v[0], c.v[1], c.v[2]);
        w = TVector3(c.w[0], c.w[1], c.w[2]);
        distance = c.distance;
        width = (int)c.width;
        height = (int)c.height;
    }
};
