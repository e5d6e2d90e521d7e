// Query dispatch of a GPU scene: the binary reference-order kernels or the
// wide/quantised fast path, the host-array path, and keeping the derived wide
// tree in step with refits.
#include <algorithm>

#include "scene.h"

namespace fcpwgb {

cudaError_t launchWide(int W, int bits, int dim, bool precise, const WideLaunch &l, cudaStream_t s) {
    switch (W) {
        case 2: return launchWideClosestT<2>(bits, dim, precise, l, s);
        case 4: return launchWideClosestT<4>(bits, dim, precise, l, s);
        default: return launchWideClosestT<8>(bits, dim, precise, l, s);
    }
}

cudaError_t launchWideRays(int W, int bits, int dim, const WideRayLaunch &l, cudaStream_t s) {
    switch (W) {
        case 2: return launchWideRayT<2>(bits, dim, l, s);
        case 4: return launchWideRayT<4>(bits, dim, l, s);
        default: return launchWideRayT<8>(bits, dim, l, s);
    }
}

namespace {
cudaError_t launchRequant(int W, int bits, unsigned char *wn, const int32_t *cb, const unsigned char *bn, int stride,
                          uint32_t n, uint32_t *err, cudaStream_t s) {
    switch (W) {
        case 2: return launchRequantizeT<2>(bits, wn, cb, bn, stride, n, err, s);
        case 4: return launchRequantizeT<4>(bits, wn, cb, bn, stride, n, err, s);
        default: return launchRequantizeT<8>(bits, wn, cb, bn, stride, n, err, s);
    }
}
}  // namespace

int GpuScene::ensureWide(cudaStream_t st) {
    const WideConfig &c = wideConfig;
    if (wide.valid && wide.branching == c.branching && wide.bits == c.bits && wide.leafSize == c.leafSize) return 0;
    // invalid until the rebuild completes: a failed allocation releases the old buffers
    wide.valid = false;
    WideHost h;
    const WideHost *pre = nullptr;
    for (const auto &p : preloadedWide)
        if (p.second.W == c.branching && p.second.bits == c.bits && p.first == c.leafSize) pre = &p.second;
    if (pre) {
        h = *pre;  // read from a scene file: no collapse
    } else if (!buildWideTree(c.branching, c.bits, hostNP, hostOff, hostBoxes, h, c.leafSize)) {
        return setError(FCPWGB_ERR_UNSUPPORTED, "this tree cannot be collapsed into the requested wide layout");
    }
    int rc;
    if ((rc = wideNodes.upload(h.nodes.data(), h.nodes.size(), st))) return rc;
    if ((rc = wideChildBinary.upload(h.childBinary.data(), h.childBinary.size() * sizeof(int32_t), st))) return rc;
    cudaError_t e;
    if (dim == 3) {
        if ((rc = widePrims.ensure((size_t)nPrims * 48))) return rc;
        if ((e = launchPackTri48((const DevTriangle *)prims.ptr, nPrims, (float4 *)widePrims.ptr, st)) != cudaSuccess)
            return cudaFail(e, "pack triangles");
    }
    // the host boxes are those of the transfer; the device tree may have been refit since
    if ((e = launchRequant(c.branching, c.bits, (unsigned char *)wideNodes.ptr, (const int32_t *)wideChildBinary.ptr,
                           (const unsigned char *)nodes.ptr, snch ? 64 : 32, h.nNodes, (uint32_t *)errorWord.ptr,
                           st)) != cudaSuccess)
        return cudaFail(e, "requantize");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "wide build");
    wide.valid = true;
    wide.branching = c.branching;
    wide.bits = c.bits;
    wide.leafSize = c.leafSize;
    wide.nNodes = h.nNodes;
    wide.depth = h.depth;
    wide.builtFromVersion = treeVersion;
    smCount();
    return 0;
}

int GpuScene::smCount() {
    if (numSMs == 0) {
        cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, device);
        if (numSMs <= 0) numSMs = 1;
    }
    return numSMs;
}

int GpuScene::wideClosest(const DevSphere *spheres, DevInteraction *out, uint32_t n, int recordNormal,
                          unsigned long long *stats, cudaStream_t st, uint32_t *inv) {
    int rc = ensureWide(st);
    if (rc) return rc;
    if (n == 0) return 0;
    const WideConfig &c = wideConfig;
    WideLaunch l;
    l.nodes = (const unsigned char *)wideNodes.ptr;
    l.prims = dim == 3 ? (const unsigned char *)widePrims.ptr : (const unsigned char *)prims.ptr;
    l.spheres = spheres;
    l.out = out;
    l.n = n;
    l.recordNormal = recordNormal;
    l.errorWord = (uint32_t *)errorWord.ptr;
    l.stats = stats;
    cudaError_t e;
    if (c.sortQueries && n >= 4096) {
        if ((rc = sortCells.ensure(sizeof(uint32_t) * kSortScratchWords))) return rc;
        if ((rc = sortPerm.ensure((size_t)n * sizeof(uint32_t)))) return rc;
        if ((rc = sortSpheres.ensure((size_t)n * sizeof(DevSphere)))) return rc;
        if ((e = launchSortQueries(sortLimits(), spheres, n, (uint32_t *)sortCells.ptr, (DevSphere *)sortSpheres.ptr,
                                   (uint32_t *)sortPerm.ptr, numSMs, st, inv)) != cudaSuccess)
            return cudaFail(e, "sort queries");
        l.spheres = (const DevSphere *)sortSpheres.ptr;
        l.perm = (const uint32_t *)sortPerm.ptr;
        l.deferRefine = inv != nullptr;
    }
    if (c.precise && dim == 3) {
        if ((rc = refineSel.ensure((size_t)n * sizeof(uint2)))) return rc;
        l.sel = (uint2 *)refineSel.ptr;
    }
    uint32_t blocks = (n + 127) / 128;
    l.packet = c.packet;
    l.shortStack = c.shortStack;
    l.lanes = c.lanes;
    if (c.persistent && c.lanes == 1) {  // persistent threads, or packets fed to warps from a counter
        if ((rc = workCounter.ensure(16))) return rc;
        if ((e = cudaMemsetAsync(workCounter.ptr, 0, 4, st)) != cudaSuccess) return cudaFail(e, "memset");
        l.counter = (uint32_t *)workCounter.ptr;
        blocks = std::min<uint32_t>(blocks, (uint32_t)numSMs * 8u);  // one resident wave
    }
    l.grid = blocks;
    if (!stats && (rc = timeStart(st))) return rc;
    if ((e = launchWide(c.branching, c.bits, dim, c.precise != 0, l, st)) != cudaSuccess)
        return cudaFail(e, "wide closest point launch");
    return stats ? 0 : timeEnd(st);
}

// the sort grid covers the queries, but no more than the scene box grown by
// twice its largest extent on every side
SortLimits GpuScene::sortLimits() const {
    float ext = 1e-6f;
    for (int a = 0; a < dim; a++) ext = std::max(ext, rootBox[3 + a] - rootBox[a]);
    SortLimits g;
    g.lo = make_float3(rootBox[0] - 2.0f * ext, rootBox[1] - 2.0f * ext, rootBox[2] - 2.0f * ext);
    g.hi = make_float3(rootBox[3] + 2.0f * ext, rootBox[4] + 2.0f * ext, rootBox[5] + 2.0f * ext);
    g.dim = dim;
    return g;
}

int GpuScene::wideRays(const DevRay *r, DevInteraction *out, uint32_t n, int occl, cudaStream_t st) {
    int rc = ensureWide(st);
    if (rc) return rc;
    if (n == 0) return 0;
    WideRayLaunch l;
    l.nodes = (const unsigned char *)wideNodes.ptr;
    l.prims = dim == 3 ? (const unsigned char *)widePrims.ptr : (const unsigned char *)prims.ptr;
    l.rays = r;
    l.out = out;
    l.n = n;
    l.occl = occl;
    l.packet = wideConfig.packet;
    l.errorWord = (uint32_t *)errorWord.ptr;
    cudaError_t e;
    // per-lane refill reads the rays in the caller's order: on 4M random rays it took 0.76 ms unsorted
    // against 1.25 ms with the octant-and-origin sort (0.45 ms of it the sort itself)
    const bool refill = wideConfig.persistent && !wideConfig.packet;
    if (refill) {  // per-lane refill from a counter, one resident wave
        if ((rc = workCounter.ensure(16))) return rc;
        if ((e = cudaMemsetAsync(workCounter.ptr, 0, 4, st)) != cudaSuccess) return cudaFail(e, "memset");
        l.counter = (uint32_t *)workCounter.ptr;
        l.grid = std::min<uint32_t>((n + 127) / 128, (uint32_t)smCount() * 8u);
    }
    if (wideConfig.sortQueries && !refill && n >= 4096) {
        if ((rc = sortCells.ensure(sizeof(uint32_t) * kSortScratchWords))) return rc;
        if ((rc = sortPerm.ensure((size_t)n * sizeof(uint32_t)))) return rc;
        if ((rc = sortRays.ensure((size_t)n * sizeof(DevRay)))) return rc;
        if ((e = launchSortRays(sortLimits(), r, n, (uint32_t *)sortCells.ptr, (DevRay *)sortRays.ptr,
                                (uint32_t *)sortPerm.ptr, numSMs, st, true)) != cudaSuccess)
            return cudaFail(e, "sort rays");
        l.rays = (const DevRay *)sortRays.ptr;
        l.perm = (const uint32_t *)sortPerm.ptr;
        l.callerRays = r;
        l.sortInfo = (const int *)((const uint32_t *)sortCells.ptr + kSortCells);
    }
    if ((rc = timeStart(st))) return rc;
    if ((e = launchWideRays(wideConfig.branching, wideConfig.bits, dim, l, st)) != cudaSuccess)
        return cudaFail(e, "wide ray launch");
    return timeEnd(st);
}

int GpuScene::timeStart(cudaStream_t st) {
    if (!timing) return 0;
    std::pair<cudaEvent_t, cudaEvent_t> p;
    if (!freeEvents.empty()) {
        p = freeEvents.back();
        freeEvents.pop_back();
    } else {
        cudaError_t e = cudaEventCreate(&p.first);
        if (e == cudaSuccess) e = cudaEventCreate(&p.second);
        if (e != cudaSuccess) return cudaFail(e, "cudaEventCreate");
    }
    timedEvents.push_back(p);
    cudaError_t e = cudaEventRecord(p.first, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "cudaEventRecord");
}

int GpuScene::timeEnd(cudaStream_t st) {
    if (!timing || timedEvents.empty()) return 0;
    cudaError_t e = cudaEventRecord(timedEvents.back().second, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "cudaEventRecord");
}

int GpuScene::closestPoints(const DevSphere *spheres, DevInteraction *out, uint32_t n, int recordNormal,
                            cudaStream_t st) {
    if (useWide()) return wideClosest(spheres, out, n, recordNormal, nullptr, st);
    int rc = timeStart(st);
    if (rc) return rc;
    cudaError_t e = launchClosestPointBinary(view(), spheres, out, n, recordNormal, st);
    if (e != cudaSuccess) return cudaFail(e, "closest point launch");
    return timeEnd(st);
}

int GpuScene::closestPointsStats(const DevSphere *spheres, DevInteraction *out, uint32_t n,
                                 unsigned long long *stats, cudaStream_t st) {
    if (useWide()) return wideClosest(spheres, out, n, 0, stats, st);
    cudaError_t e = launchClosestPointBinaryStats(view(), spheres, out, n, stats, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "closest point stats launch");
}

int GpuScene::rays(const DevRay *r, DevInteraction *out, uint32_t n, int occl, cudaStream_t st) {
    if (useWide()) return wideRays(r, out, n, occl, st);
    cudaError_t e = launchRayBinary(view(), r, out, n, occl, st);
    return e == cudaSuccess ? 0 : cudaFail(e, "ray launch");
}

// The device address of a caller's page-locked host array (cudaHostAlloc, or
// registered mapped), NULL for pageable memory.
static void *mappedHostPointer(void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory on older runtimes: not an error of ours
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int GpuScene::closestPointsHost(const fcpwgb_bounding_sphere *spheres, fcpwgb_interaction *out, uint32_t n,
                                int recordNormal) {
    size_t ib = (size_t)n * sizeof(DevSphere), ob = (size_t)n * sizeof(DevInteraction);
    int rc;
    if ((rc = qIn0.ensure(ib))) return rc;
    if ((rc = qOut.ensure(ob))) return rc;
    cudaError_t e = cudaMemcpyAsync(qIn0.ptr, spheres, ib, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    // Precise mode on triangles with sorted queries, into a page-locked array:
    // the refinement pass runs in the caller's order and writes each record
    // straight into the caller's array over the host link, coalesced, instead
    // of a device buffer copied back afterwards (the copy would follow the pass;
    // this way the pass's work hides under the transfer). The same records.
    DevInteraction *direct = nullptr;
    if (useWide() && wideConfig.precise && dim == 3 && wideConfig.sortQueries && n >= 4096 && !inst)
        direct = (DevInteraction *)mappedHostPointer(out);
    if (((uintptr_t)direct & 15u) != 0) direct = nullptr;  // the pass stores 16 B vectors from the array's start
    if (direct) {
        if ((rc = sortInv.ensure((size_t)n * sizeof(uint32_t)))) return rc;
        if ((rc = wideClosest((const DevSphere *)qIn0.ptr, (DevInteraction *)qOut.ptr, n, recordNormal, nullptr, stream,
                              (uint32_t *)sortInv.ptr)))
            return rc;
        if ((e = launchRefineTrianglesInOrder((const unsigned char *)widePrims.ptr, (const DevSphere *)qIn0.ptr,
                                              (const uint32_t *)sortInv.ptr, (const uint2 *)refineSel.ptr, direct, n,
                                              recordNormal, stream)) != cudaSuccess)
            return cudaFail(e, "refinement in the caller's order");
    } else {
        if ((rc = closestPoints((const DevSphere *)qIn0.ptr, (DevInteraction *)qOut.ptr, n, recordNormal, stream)))
            return rc;
        e = cudaMemcpyAsync(out, qOut.ptr, ob, cudaMemcpyDeviceToHost, stream);
        if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    }
    uint32_t err[4] = {0, 0, 0, 0};
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

int GpuScene::containsPoints(const float *points, uint32_t n, uint32_t *result, cudaStream_t st) {
    cudaError_t e;
    if (useWide() && wideConfig.sortQueries && n >= 4096) {
        // the rays of contains go along +x and +y from every point: sorted points
        // walk the tree alike; each point's answer is unchanged
        int rc;
        if ((rc = packedPoints.ensure((size_t)n * sizeof(DevSphere))) ||
            (rc = sortCells.ensure(sizeof(uint32_t) * kSortScratchWords)) ||
            (rc = sortPerm.ensure((size_t)n * sizeof(uint32_t))) ||
            (rc = sortSpheres.ensure((size_t)n * sizeof(DevSphere))))
            return rc;
        if ((e = launchPackPoints(points, n, (DevSphere *)packedPoints.ptr, st)) != cudaSuccess)
            return cudaFail(e, "pack points");
        if ((e = launchSortQueries(sortLimits(), (const DevSphere *)packedPoints.ptr, n, (uint32_t *)sortCells.ptr,
                                   (DevSphere *)sortSpheres.ptr, (uint32_t *)sortPerm.ptr, smCount(), st)) != cudaSuccess)
            return cudaFail(e, "sort points");
        if ((e = launchContains(view(), (const float *)sortSpheres.ptr, 4, (const uint32_t *)sortPerm.ptr, n, result,
                                st)) != cudaSuccess)
            return cudaFail(e, "contains");
        return 0;
    }
    if ((e = launchContains(view(), points, 3, nullptr, n, result, st)) != cudaSuccess) return cudaFail(e, "contains");
    return 0;
}

int GpuScene::afterRefit(cudaStream_t st) {
    if (!wide.valid) return 0;
    cudaError_t e;
    if (dim == 3 && (e = launchPackTri48((const DevTriangle *)prims.ptr, nPrims, (float4 *)widePrims.ptr, st)) !=
                        cudaSuccess)
        return cudaFail(e, "pack triangles");
    if ((e = launchRequant(wide.branching, wide.bits, (unsigned char *)wideNodes.ptr,
                           (const int32_t *)wideChildBinary.ptr, (const unsigned char *)nodes.ptr, snch ? 64 : 32,
                           wide.nNodes, (uint32_t *)errorWord.ptr, st)) != cudaSuccess)
        return cudaFail(e, "requantize");
    return 0;
}

}  // namespace fcpwgb
