// Per-vertex tangents of Model::generateTangents (model.cpp:430-476) on the GPU,
// for the models whose tangents the loader leaves to the device (every model
// with the generateTangent flag that is not normalised; fr_scene.cpp).
//
// The reference runs one loop per model: for each mesh (map key order) and each
// face, the face's tangent (its operation order, float) is added to the running
// sums of its three corners; then every sum is normalised, (1, 0, 0) where it is
// zero. Each vertex's sum is a float sum in face order, so the device keeps that
// order instead of scattering with atomics: the (vertex, face) pairs are listed
// face by face and stably sorted by vertex, which puts each vertex's faces in
// draw order (the scene's global triangle order restricted to one model is the
// loop's order), and one thread per vertex adds them in sequence.
#include <cub/cub.cuh>

#include <vector>

#include "fr_context_internal.h"
#include "fr_device.cuh"

namespace
{
using namespace frd;

// One face's tangent, or w = 0 where the reference skips the face (det == 0).
__global__ void k_face_tangent(const float4* __restrict__ pos, const float2* __restrict__ uv,
                               const int4* __restrict__ triV, const int4* __restrict__ triT,
                               const int* __restrict__ faces, int nf, float4* __restrict__ faceT,
                               int* __restrict__ keys, int* __restrict__ vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const int f = faces[i];
    const int4 v = triV[f], t = triT[f];
    keys[3 * i] = v.x, keys[3 * i + 1] = v.y, keys[3 * i + 2] = v.z;
    vals[3 * i] = vals[3 * i + 1] = vals[3 * i + 2] = i;
    const float4 p0 = pos[v.x], p1 = pos[v.y], p2 = pos[v.z];
    const float2 t0 = uv[t.x], t1 = uv[t.y], t2 = uv[t.z];
    const F3 e1{p1.x - p0.x, p1.y - p0.y, p1.z - p0.z}, e2{p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
    const float d1s = t1.x - t0.x, d1t = t1.y - t0.y, d2s = t2.x - t0.x, d2t = t2.y - t0.y;
    const float det = d1s * d2t - d2s * d1t;
    if (det == 0.f)
    {
        faceT[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float inv = 1.f / det;
    const F3 raw{d2t * e1.x - d1t * e2.x, d2t * e1.y - d1t * e2.y, d2t * e1.z - d1t * e2.z};
    const F3 T = normalize(raw * inv);
    faceT[i] = make_float4(T.x, T.y, T.z, 1.f);
}

// The first index in sorted keys[0, n) holding a value >= v.
__device__ __forceinline__ int lower_bound(const int* __restrict__ keys, int n, int v)
{
    int lo = 0, hi = n;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// One vertex of a pending model: its faces' tangents summed in draw order, normalised.
__global__ void k_vertex_tangent(const int* __restrict__ vmodel, const unsigned char* __restrict__ pending, int nv,
                                 const int* __restrict__ keys, const int* __restrict__ vals, int npairs,
                                 const float4* __restrict__ faceT, float4* __restrict__ tan)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv || !pending[vmodel[v]]) return;
    F3 acc{0.f, 0.f, 0.f};
    for (int j = lower_bound(keys, npairs, v); j < npairs && keys[j] == v; ++j)
    {
        const float4 T = faceT[vals[j]];
        if (T.w != 0.f) acc = acc + F3{T.x, T.y, T.z};
    }
    const F3 t = length(acc) == 0.f ? F3{1.f, 0.f, 0.f} : normalize(acc);
    tan[v] = make_float4(t.x, t.y, t.z, 0.f);
}

}  // namespace

// Tangents of the pending models into S.tan (the rest of S.tan as uploaded).
// faces: the pending models' triangles in draw order. Synchronous; allocates
// its scratch for the call.
int fr_generate_tangents(fr_ctx* ctx, const std::vector<int>& faces, const std::vector<unsigned char>& pendingModels)
{
    const frd::DevScene& S = ctx->S;
    const int nf = (int)faces.size(), np = 3 * nf, nv = S.numVerts;
    cudaStream_t st = ctx->stream;
    std::vector<void*> bufs;
    auto get = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return p;
    };
    auto done = [&](int rc) {
        cudaStreamSynchronize(st);
        for (void* p : bufs) cudaFree(p);
        return rc;
    };
    int* dFaces = (int*)get(sizeof(int) * (size_t)nf);
    float4* faceT = (float4*)get(sizeof(float4) * (size_t)nf);
    int* keys = (int*)get(sizeof(int) * (size_t)np);
    int* vals = (int*)get(sizeof(int) * (size_t)np);
    int* keys2 = (int*)get(sizeof(int) * (size_t)np);
    int* vals2 = (int*)get(sizeof(int) * (size_t)np);
    unsigned char* dPending = (unsigned char*)get(pendingModels.size());
    if (!dFaces || !faceT || !keys || !vals || !keys2 || !vals2 || !dPending) return done(FR_ERR_CUDA);
    if (cudaMemcpyAsync(dFaces, faces.data(), sizeof(int) * (size_t)nf, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dPending, pendingModels.data(), pendingModels.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return done(FR_ERR_CUDA);
    if (nf > 0)
        k_face_tangent<<<(nf + 255) / 256, 256, 0, st>>>(S.pos, S.uv, S.triV, S.triT, dFaces, nf, faceT, keys, vals);
    int bits = 1;
    while (bits < 31 && (1 << bits) < nv) ++bits;
    size_t tmpBytes = 0;
    if (np > 0)
    {
        // LSD radix sort: stable, so each vertex's pairs keep their face order
        cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, keys, keys2, vals, vals2, np, 0, bits, st);
        void* tmp = get(tmpBytes);
        if (!tmp) return done(FR_ERR_CUDA);
        if (cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keys, keys2, vals, vals2, np, 0, bits, st) != cudaSuccess)
            return done(FR_ERR_CUDA);
    }
    if (nv > 0)
        k_vertex_tangent<<<(nv + 255) / 256, 256, 0, st>>>(S.vmodel, dPending, nv, keys2, vals2, np, faceT,
                                                            const_cast<float4*>(S.tan));
    if (cudaGetLastError() != cudaSuccess) return done(FR_ERR_CUDA);
    return done(cudaStreamSynchronize(st) == cudaSuccess ? FR_OK : FR_ERR_CUDA);
}
