// dataterm.cuh -- host launchers of the batched data-term kernels.
#pragma once

#include "engine.cuh"

namespace gcfg {

constexpr int NBINS = 4096;                   // 16^3 colour bins per class
#ifndef GCFG_CHUNK_PX
// batch256 histogram/sigma pass: 0.159 / 0.128 / 0.118 / 0.143 ms at 2K / 4K / 8K / 16K pixels per
// chunk; 8K leaves a single 1920x1080 image too few blocks (0.021 -> 0.032 ms), so 4K it is
#define GCFG_CHUNK_PX 4096
#endif
constexpr int CHUNK_PX = GCFG_CHUNK_PX;       // pixels per block in per-image passes (about)

// Rows of a W-wide image per block of the histogram / sigma pass.
// Blocks of the per-image pass over an image: CHUNK_PX consecutive pixels
// (row-major) each, the last one shorter.
inline long long image_chunks(int W, int H) { return ((long long)W * H + CHUNK_PX - 1) / CHUNK_PX; }

// Device buffers of the data term for a batch (per image: 2*4096 histogram
// bins, 4096 dp and dn entries).
struct DtArgs {
    int n_img;                // images of this pass (local index k)
    const int *ilist;         // local image k -> image (slot) index; NULL: k itself
    long long total_chunks;
    const uint8_t *rgb;       // packed row-major RGB of all images
    const uint8_t *scrib;     // packed row-major scribbles (0 none, 1 fg, 2 bg)
    const ImgDesc *img;
    ImgState *ist;
    const int2 *chunk_map;    // per chunk of the pass: (image index, chunk index within the image)
    int *hist;
    int *dp_lut, *dn_lut;
    double *raw_dp, *raw_dn;  // optional (NULL): pre-rounding per-bin values
};

gcfg_status dt_tables(const DtArgs &a, cudaStream_t st);
gcfg_status dt_build(const Batch &b, const DtArgs &a, cudaStream_t st);
gcfg_status dt_apply_tlinks(const DtArgs &a, long long n, int *dp, int *dn, cudaStream_t st);
gcfg_status dt_apply_nlinks(const DtArgs &a, int W, int H, int *up, int *down, int *left, int *right,
                            cudaStream_t st);

}  // namespace gcfg
