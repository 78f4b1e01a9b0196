// gvx_convert.cu -- ConvertAndTransform (VG.cpp:5668-5682, kernel
// gvdbConvAndTransform PT.cuh:120-142): the point decode the point-cloud
// callers run before SetPoints.  Each point (three uint16 when src_bits is 2,
// three floats when 4) becomes float3 (wmin + p * wdelta) * scal + trans,
// written densely (12-byte stride) whatever dst_bits says, as the reference
// writes it.  Both multiply-adds are single-rounding FMAs, the form the
// reference's build contracts them to.
#include "gvx_grid.cuh"

__global__ void k_convert_points(const unsigned char* __restrict__ src, int src_bits, float* __restrict__ dst,
                                 uint32_t n, float3 wmin, float3 wdelta, float3 trans, float3 scal)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float p[3];
        if (src_bits == 2) {
            const unsigned short* s = (const unsigned short*)(src + (size_t)i * 6);
            p[0] = (float)s[0];
            p[1] = (float)s[1];
            p[2] = (float)s[2];
        } else {
            const float* s = (const float*)(src + (size_t)i * 12);
            p[0] = s[0];
            p[1] = s[1];
            p[2] = s[2];
        }
        const float mn[3] = {wmin.x, wmin.y, wmin.z}, dl[3] = {wdelta.x, wdelta.y, wdelta.z};
        const float sc[3] = {scal.x, scal.y, scal.z}, tr[3] = {trans.x, trans.y, trans.z};
#pragma unroll
        for (int a = 0; a < 3; a++) dst[(size_t)i * 3 + a] = __fmaf_rn(__fmaf_rn(p[a], dl[a], mn[a]), sc[a], tr[a]);
    }
}

extern "C" gvx_status gvx_convert_and_transform(gvx_grid* g, const void* src, int src_bits, void* dst, int dst_bits,
                                                int n, const float wmin[3], const float wdelta[3],
                                                const float trans[3], const float scal[3])
{
    if (!g) {
        gvx_set_error("null grid handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    (void)dst_bits;  // the reference writes float3 whatever it says (PT.cuh:141)
    if (n < 0 || (n > 0 && (!src || !dst)) || !wmin || !wdelta || !trans || !scal) {
        gvx_set_error("ConvertAndTransform: %d points, null buffer or vector", n);
        return GVX_ERR_INVALID_ARG;
    }
    if (src_bits != 2 && src_bits != 4) {
        gvx_set_error("ConvertAndTransform: source format %d (2 = uint16 x3, 4 = float x3)", src_bits);
        return GVX_ERR_INVALID_ARG;
    }
    if (((uintptr_t)dst & 3) || (src_bits == 4 && ((uintptr_t)src & 3)) || ((uintptr_t)src & 1)) {
        gvx_set_error("ConvertAndTransform: misaligned buffer");
        return GVX_ERR_INVALID_ARG;
    }
    if (n == 0) return GVX_OK;
    const unsigned threads = 256;
    const unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)n + threads - 1) / threads, 152ull * 16ull);
    k_convert_points<<<blocks, threads, 0, g->stream>>>(
        (const unsigned char*)src, src_bits, (float*)dst, (uint32_t)n, make_float3(wmin[0], wmin[1], wmin[2]),
        make_float3(wdelta[0], wdelta[1], wdelta[2]), make_float3(trans[0], trans[1], trans[2]),
        make_float3(scal[0], scal[1], scal[2]));
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
