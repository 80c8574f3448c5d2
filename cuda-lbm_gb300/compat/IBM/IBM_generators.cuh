// lbmx compat: marker generators a scenario may call
// (create_cylinder, src/IBM/IBM_generators.cuh:8, IBM_generators.cu:5-25):
// num_pts markers evenly spaced on a circle, starting at angle 0.
#ifndef IBM_GENERATORS_H
#define IBM_GENERATORS_H
#include <math.h>

#include "IBM/IBMBody.cuh"

inline IBMBody create_cylinder(float cx, float cy, float r, int num_pts = 16) {
    IBMBody body{num_pts, new float[2 * num_pts], new float[2 * num_pts]};
    const double step = 2.0 * 3.14159265358979323846 / num_pts;
    for (int i = 0; i < num_pts; i++) {
        body.points[2 * i] = cx + r * (float)cos(i * step);
        body.points[2 * i + 1] = cy + r * (float)sin(i * step);
        body.velocities[2 * i] = 0.0f;
        body.velocities[2 * i + 1] = 0.0f;
    }
    return body;
}

#endif
