// Query dispatch of a GPU scene: picks the traversal variant and runs the
// host-array path.
#include "scene.h"

namespace fcpwgb {

int GpuScene::closestPoints(const DevSphere *spheres, DevInteraction *out, uint32_t n, int recordNormal,
                            cudaStream_t st) {
    cudaError_t e = launchClosestPointBinary(view(), spheres, out, n, recordNormal, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "closest point launch");
}

int GpuScene::closestPointsStats(const DevSphere *spheres, DevInteraction *out, uint32_t n,
                                 unsigned long long *stats, cudaStream_t st) {
    cudaError_t e = launchClosestPointBinaryStats(view(), spheres, out, n, stats, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "closest point stats launch");
}

int GpuScene::rays(const DevRay *r, DevInteraction *out, uint32_t n, int occl, cudaStream_t st) {
    cudaError_t e = launchRayBinary(view(), r, out, n, occl, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "ray launch");
}

int GpuScene::closestPointsHost(const fcpwgb_bounding_sphere *spheres, fcpwgb_interaction *out, uint32_t n,
                                int recordNormal) {
    size_t ib = (size_t)n * sizeof(DevSphere), ob = (size_t)n * sizeof(DevInteraction);
    int rc;
    if ((rc = qIn0.ensure(ib))) return rc;
    if ((rc = qOut.ensure(ob))) return rc;
    cudaError_t e = cudaMemcpyAsync(qIn0.ptr, spheres, ib, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    if ((rc = closestPoints((const DevSphere *)qIn0.ptr, (DevInteraction *)qOut.ptr, n, recordNormal, stream)))
        return rc;
    uint32_t err[4] = {0, 0, 0, 0};
    e = cudaMemcpyAsync(out, qOut.ptr, ob, cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    e = cudaMemcpyAsync(err, errorWord.ptr, sizeof(err), cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaStreamSynchronize");
    if (err[0]) {
        cudaMemsetAsync(errorWord.ptr, 0, sizeof(err), stream);
        cudaStreamSynchronize(stream);
        return setError(FCPWGB_ERR_TRAVERSAL, "device traversal error word " + std::to_string(err[0]));
    }
    return 0;
}

int GpuScene::afterRefit(cudaStream_t st) {
    (void)st;
    wide.clear();
    return 0;
}

}  // namespace fcpwgb
