// hw_sampler.cu — TEST INFRASTRUCTURE ONLY: decodes BC blocks in this GPU's
// texture sampler, the checker of the library's block decoder
// (wavefrontpathtracing_gb300/csrc/wf_texture.cu) and of the oracle's
// (oracle/orc_bc.c).  The reference hands DDS blocks to D3D12 as DXGI BC
// formats (core/assets/asset_loader.cpp:179-206, renderer/d3d12/
// d3d12_backend.cpp:725-740), so the texture hardware is what decodes them
// there too.
//
// The blocks go into a CUDA array of 32-bit unsigned elements (two channels
// for 8-byte blocks, four for 16-byte ones), one element per block, viewed
// through a block-compressed resource view four times as wide and high; a
// kernel reads every texel with point sampling at its centre (the view's
// element type, normalised floats).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

namespace {

__global__ void k_fetch(cudaTextureObject_t tex, uint32_t w, uint32_t h, float4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const uint32_t x = i % w, y = i / w;
    out[i] = tex2D<float4>(tex, (float)x + 0.5f, (float)y + 0.5f);
}

int report(char* err, int len, const char* what, cudaError_t e) {
    if (err && len > 0) snprintf(err, (size_t)len, "%s: %s", what, cudaGetErrorString(e));
    return (int)e;
}

}  // namespace

// kind: 1..5 = BC1..BC5, 7 = BC7 (unsigned, linear); blocks: bw x bh blocks
// as a DDS file stores them; out: (4 bh) x (4 bw) x 4 floats in [0, 1].
// Returns 0 or a CUDA error code (err receives a message).
extern "C" int hws_decode_bc(int kind, const void* blocks, uint32_t bw, uint32_t bh, float* out, char* err,
                             int err_len) {
    cudaResourceViewFormat view;
    switch (kind) {
        case 1: view = cudaResViewFormatUnsignedBlockCompressed1; break;
        case 2: view = cudaResViewFormatUnsignedBlockCompressed2; break;
        case 3: view = cudaResViewFormatUnsignedBlockCompressed3; break;
        case 4: view = cudaResViewFormatUnsignedBlockCompressed4; break;
        case 5: view = cudaResViewFormatUnsignedBlockCompressed5; break;
        case 7: view = cudaResViewFormatUnsignedBlockCompressed7; break;
        default: return report(err, err_len, "hws_decode_bc: kind", cudaErrorInvalidValue);
    }
    if (!blocks || !out || bw == 0 || bh == 0 || bw > 4096 || bh > 4096)
        return report(err, err_len, "hws_decode_bc: arguments", cudaErrorInvalidValue);
    const bool small = kind == 1 || kind == 4;
    const size_t block_bytes = small ? 8 : 16;
    const cudaChannelFormatDesc desc =
        small ? cudaCreateChannelDesc(32, 32, 0, 0, cudaChannelFormatKindUnsigned)
              : cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindUnsigned);
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    float4* d_out = nullptr;
    const uint32_t w = 4 * bw, h = 4 * bh;
    cudaError_t e = cudaMallocArray(&arr, &desc, bw, bh);
    if (e != cudaSuccess) return report(err, err_len, "cudaMallocArray", e);
    e = cudaMemcpy2DToArray(arr, 0, 0, blocks, bw * block_bytes, bw * block_bytes, bh, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;   // the BC view reads as normalised floats
        td.normalizedCoords = 0;
        cudaResourceViewDesc vd = {};
        vd.format = view;
        vd.width = w;
        vd.height = h;
        e = cudaCreateTextureObject(&tex, &rd, &td, &vd);
        if (e != cudaSuccess) report(err, err_len, "cudaCreateTextureObject", e);
    } else {
        report(err, err_len, "cudaMemcpy2DToArray", e);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&d_out, (size_t)w * h * sizeof(float4));
        if (e != cudaSuccess) report(err, err_len, "cudaMalloc", e);
    }
    if (e == cudaSuccess) {
        k_fetch<<<(w * h + 255) / 256, 256>>>(tex, w, h, d_out);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(out, d_out, (size_t)w * h * sizeof(float4), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) report(err, err_len, "fetch", e);
    }
    if (tex) cudaDestroyTextureObject(tex);
    if (d_out) cudaFree(d_out);
    cudaFreeArray(arr);
    return (int)e;
}
