// ##################################################################
//
// api_internal.h -- solver-handle construction shared by the C ABI
// (api.cu) and the host classes (host/hamstr_host.cpp)
// ##################################################################
#ifndef HAMSTR_GPU_API_INTERNAL_H
#define HAMSTR_GPU_API_INTERNAL_H

#include <string>
#include <vector>

#include "../../include/hamstr_gpu.h"

namespace hamstr {

// Instances of a batched handle: a disjoint union of meshes, instance k
// owning cells cell0[k]..cell0[k+1]-1 and chains chain0[k]..chain0[k+1]-1,
// with its own freestream (rinf uinf vinf einf, 4 per instance).
struct InstanceInfo {
   int n = 1;
   std::vector<int> cell0, chain0;
   std::vector<double> freestream;
};

// message returned by hamstr_gpu_last_error
void set_last_error(const std::string& m);

// hamstr_gpu_create with instances (nullptr: one instance, p's freestream)
int create_gpu(const hamstr_gpu_params* p, int nCell, int nFace, const int* faces, const double* normVec,
               const double* refMtx, int nChain, const int* faceStartPerChain, const int* chainConn,
               const InstanceInfo* inst, hamstr_gpu** out);

}  // namespace hamstr
#endif
