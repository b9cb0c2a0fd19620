// Host build of the reference's packed-site decoder (backends/metal/shaders/sad_common.metal:
// PackedSiteQuant, PackedInferenceSite, unpackUnorm16, packedActive, decodePackedSite),
// compiled from its source under metal_shim.h by oracle/ref/metal_decode.py.  It decodes
// words the way the reference's packed renderers call it (sad_common.metal:355, dims =
// (width - 1, height - 1), packed_render_encoder.metal:16).  Test infrastructure only.
#include "metal_shim.h"
#include "metal_decode_slice.h"  // generated into oracle/_ref from the reference's source

extern "C" void ref_decode_packed(const uint32_t* words, const float* quant10, int n, int width, int height,
                                  float* out10, int* active) {
    PackedSiteQuant q;
    static_assert(sizeof(PackedSiteQuant) == 10 * sizeof(float), "PackedSiteQuant layout");
    std::memcpy(&q, quant10, sizeof(q));
    const float2 dims(static_cast<float>(width - 1), static_cast<float>(height - 1));
    for (int i = 0; i < n; ++i) {
        PackedInferenceSite p;
        p.data = uint4{words[4 * i], words[4 * i + 1], words[4 * i + 2], words[4 * i + 3]};
        const VoronoiSite s = decodePackedSite(p, dims, q);
        float* o = out10 + 10 * i;
        o[0] = s.position.x;
        o[1] = s.position.y;
        o[2] = s.log_tau;
        o[3] = s.radius;
        o[4] = s.color.x;
        o[5] = s.color.y;
        o[6] = s.color.z;
        o[7] = s.aniso_dir.x;
        o[8] = s.aniso_dir.y;
        o[9] = s.log_aniso;
        active[i] = packedActive(p) ? 1 : 0;
    }
}

// The packed render of renderVoronoiPacked (packed_render_encoder.metal:3-31) with a
// candidate field of the output's size: per pixel, the candidate lists c0 / c1 ([H*W][4]
// u32 each), uv = the pixel's coordinates, dims = (width - 1, height - 1); a pixel whose
// candidates are all invalid is black.
extern "C" void ref_render_packed(const uint32_t* words, const float* quant10, int n, const uint32_t* c0,
                                  const uint32_t* c1, float inv_scale_sq, int width, int height, float* rgb) {
    PackedSiteQuant q;
    std::memcpy(&q, quant10, sizeof(q));
    PackedInferenceSite* sites = new PackedInferenceSite[n > 0 ? n : 1];
    for (int i = 0; i < n; ++i)
        sites[i].data = uint4{words[4 * i], words[4 * i + 1], words[4 * i + 2], words[4 * i + 3]};
    const float2 dims(static_cast<float>(width - 1), static_cast<float>(height - 1));
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            const size_t p = static_cast<size_t>(y) * width + x;
            uint ids[8];
            for (int k = 0; k < 4; ++k) {
                ids[k] = c0[4 * p + k];
                ids[4 + k] = c1[4 * p + k];
            }
            float weights[8];
            float3 pred;
            const bool ok = computePackedWeights(ids, sites, q, static_cast<uint>(n),
                                                 float2(static_cast<float>(x), static_cast<float>(y)), inv_scale_sq,
                                                 dims, weights, pred);
            rgb[3 * p] = ok ? pred.x : 0.0f;
            rgb[3 * p + 1] = ok ? pred.y : 0.0f;
            rgb[3 * p + 2] = ok ? pred.z : 0.0f;
        }
    delete[] sites;
}
