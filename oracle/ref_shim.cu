// ref_shim.cu -- TEST INFRASTRUCTURE.  Link-time stand-ins for the device
// utility functions of the reference (declared in femmd2D/src/def.h:52-53,
// 181-185, femmd2D/src/CudaUtil.h:23-25 and redeclared in md3dsystem.cpp:144-147)
// whose original translation unit, CudaUtil.cu, does not compile under
// CUDA 13 (it reads cudaDeviceProp fields that CUDA 13 removed).  The
// reference harness only runs the reference's CPU path, so the device report
// is a no-op and the thrust helpers are plain one-line implementations of
// what their names and signatures state.
#include <thrust/device_vector.h>
#include <thrust/reduce.h>
#include <thrust/transform.h>
#include <thrust/functional.h>
#include "def.h"

void md_device_init(int, char **) {}
void md_device_report() {}
void resetDevce() {}
void cudaCopyToDevice(void *d, void *h, int size) { cudaMemcpy(d, h, size, cudaMemcpyHostToDevice); }

struct shim_norm2 {
    __host__ __device__ real operator()(const VectorR &a) const { return a.x * a.x + a.y * a.y; }
};

void squareVec(dvector<VectorR> &v, dvector<real> &vv) { thrust::transform(v.begin(), v.end(), vv.begin(), shim_norm2()); }
real findMax(dvector<real> &v) { return thrust::reduce(v.begin(), v.end(), (real)0, thrust::maximum<real>()); }
void multVec(dvector<real> &vv, dvector<real> &m) {
    thrust::transform(vv.begin(), vv.end(), m.begin(), vv.begin(), thrust::multiplies<real>());
}
real reduce(dvector<real> &vv) { return thrust::reduce(vv.begin(), vv.end()); }

template <typename T> static void shim_release(dvector<T> &v) {
    v.clear();
    dvector<T>().swap(v);
}
void clearDevVector(dvector<int> &v) { shim_release(v); }
void clearDevVector(dvector<real> &v) { shim_release(v); }
void clearDevVector(dvector<VectorR> &v) { shim_release(v); }
void clearDevVector(dvector<tetraIndexes> &v) { shim_release(v); }
void clearDevVector(dvector<mat3x3> &v) { shim_release(v); }
