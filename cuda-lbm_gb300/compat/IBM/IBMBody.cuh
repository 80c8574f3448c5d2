// lbmx compat: an IBM body as a scenario builds it (src/IBM/IBMBody.cuh):
// num_points markers, xy interleaved, host memory owned by the body.
#ifndef IBM_BODY_H
#define IBM_BODY_H

struct IBMBody {
    int num_points;
    float* points;
    float* velocities;
};

inline void h_ibm_free(IBMBody body) {
    delete[] body.points;
    delete[] body.velocities;
}

#endif
