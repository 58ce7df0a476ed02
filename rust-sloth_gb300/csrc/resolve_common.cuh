// resolve_common.cuh -- per-cell resolve shared by the single-frame and batched kernels.
//
// For every frame cell c the reference's final value is the last of three kinds of
// write in draw order (src/rasterizer.rs:80-91):
//   - the last accepted depth write at cell c          (frame_buffer[id]   = pixel)
//   - the last accepted depth write at cell c-1         (frame_buffer[id+1] = pixel)
//   - in image mode, the newline sentinel of row y when c == y*w+1
// The last accepted depth write of a cell is its minimum key.  Draw order is compared
// as (triangle, sample row, sample column); a newline comes after every sample of its
// row.  The winner's depth is its key's (the record's depth plane gives the sign of a zero
// depth), its shade and char are recomputed from its record with the raster's exact
// operations.
#pragma once

#include <climits>

#include "sloth_internal.cuh"
#include "sloth_kernels.h"

namespace sloth {

struct Cand {
    uint32_t tri;
    int32_t y, x;
    uint32_t cell;
};

__device__ __forceinline__ bool later(const Cand &a, const Cand &b)
{
    if (a.tri != b.tri) return a.tri > b.tri;
    if (a.y != b.y) return a.y > b.y;
    return a.x > b.x;
}

__device__ __forceinline__ uint64_t key_at(const FrameGeom &g, const FrameBuffers &fb, int r, int cc)
{
    // no sample writes an odd column of an even-width frame, and its key is not kept
    if (!(g.w & 1) && (cc & 1)) return kEmptyKey;
    // tile sides are powers of two; both reads issued before either is tested (the key
    // of a tile of an older generation is in bounds, only stale)
    const int tile = (r >> (__ffs(g.th) - 1)) * g.ntx + (cc >> (__ffs(g.tw) - 1));
    const uint32_t gen = __ldg(fb.tile_gen + tile);
    const uint64_t k =
        __ldg(reinterpret_cast<const unsigned long long *>(fb.keys) + (size_t)r * g.pitch + key_col(cc, g.tw));
    return gen == fb.gen ? k : kEmptyKey;
}

// decode() with the winner's record rows 0-1 already loaded (q0, q1).
__device__ __forceinline__ Cand decode_rows(const FrameGeom &g, const FrameBuffers &fb, uint64_t key, int r, int cc,
                                            float4 q0, float4 q1, float *z_out)
{
    Cand c;
    const uint32_t lo = (uint32_t)key;
    c.tri = lo >> 1;
    if (lo & 1u) {
        c.y = r;
        c.x = cc >> 1;
    } else {
        c.y = r - 1;
        c.x = (cc + g.w) >> 1;
    }
    // rows 0-1 (one 32-byte sector): vertices, shade factor, colour; the edge deltas are
    // the subtractions setup made (build_record)
    TriRecord rec;
    rec.v1x = q0.x; rec.v1y = q0.y; rec.v2x = q0.z; rec.v2y = q0.w; rec.v3x = q1.x; rec.v3y = q1.y;
    rec.dx0 = fsub(rec.v3x, rec.v2x); rec.dy0 = fsub(rec.v3y, rec.v2y);
    rec.dx1 = fsub(rec.v1x, rec.v3x); rec.dy1 = fsub(rec.v1y, rec.v3y);
    rec.dx2 = fsub(rec.v2x, rec.v1x); rec.dy2 = fsub(rec.v2y, rec.v1y);
    const EdgeVals e = eval_edges(rec, (float)c.x, (float)c.y);
    const float shade = fmul(q1.z, fadd(fadd(e.w0, e.w1), e.w2));
    if (z_out) {
        // the key holds the depth itself, except the sign of a zero (ordered_z folds -0 into
        // +0): only then the depth plane (row 5) is read and the depth recomputed
        const uint32_t hi = (uint32_t)(key >> 32);
        if (hi != ordered_z(0.0f)) {
            *z_out = float_of_ordered(hi);
        } else {
            const float4 q5 = __ldg(reinterpret_cast<const float4 *>(fb.records + c.tri) + 5);
            *z_out = interp_z(q5.x, q5.y, q5.z, q5.w, e.w1, e.w2);
        }
    }
    c.cell = shade_char(shade) | (__float_as_uint(q1.w) << 8);
    return c;
}

// Rebuild the winning write of depth cell (r, cc) from its key.
__device__ __forceinline__ Cand decode(const FrameGeom &g, const FrameBuffers &fb, uint64_t key,
                                       int r, int cc, float *z_out)
{
    const float4 *p = reinterpret_cast<const float4 *>(fb.records + ((uint32_t)key >> 1));
    return decode_rows(g, fb, key, r, cc, __ldg(p), __ldg(p + 1), z_out);
}

// Resolve frame cell c (and depth cell c when c < w*h) of one frame.
__device__ __forceinline__ void resolve_cell(const FrameGeom &g, const FrameBuffers &fb, uint64_t c)
{
    const uint64_t nz = (uint64_t)g.w * g.h;
    if (c >= nz) {
        fb.cells_out[c] = (uint32_t)' ';
        return;
    }
    const int r = (int)(c / g.w), cc = (int)(c - (uint64_t)r * g.w);
    bool have = false;
    Cand best{0, 0, 0, (uint32_t)' '};
    const uint64_t kc = key_at(g, fb, r, cc);
    if (kc != kEmptyKey) {
        float z;
        best = decode(g, fb, kc, r, cc, &z);
        have = true;
        fb.z_out[c] = z;
        fb.winner_out[c] = (int32_t)best.tri;
    } else {
        fb.z_out[c] = kFltMax;
        fb.winner_out[c] = -1;
    }
    if (c > 0) {
        const int pr = cc > 0 ? r : r - 1, pc = cc > 0 ? cc - 1 : g.w - 1;
        const uint64_t kp = key_at(g, fb, pr, pc);
        if (kp != kEmptyKey) {
            const Cand b = decode(g, fb, kp, pr, pc, nullptr);
            if (!have || later(b, best)) best = b;
            have = true;
        }
        if (g.image && (c - 1) % g.w == 0) {
            const uint64_t yn = (c - 1) / g.w;
            if (yn < (uint64_t)g.h) {
                const int32_t t = nltree_query(fb.nltree, g.nl_size, (int)yn);
                if (t >= 0) {
                    const Cand n{(uint32_t)t, (int32_t)yn, INT_MAX, (uint32_t)'\n'};
                    if (!have || later(n, best)) best = n;
                    have = true;
                }
            }
        }
    }
    fb.cells_out[c] = best.cell;
}

// The newline candidate of frame cell c (r, cc its row and column when c < w*h), if the
// frame is in image mode and c = y*w+1 for a row y some triangle spans.
__device__ __forceinline__ bool newline_at(const FrameGeom &g, const FrameBuffers &fb, uint64_t c, uint64_t nz, int r,
                                          int cc, Cand &out)
{
    if (!g.image || c == 0) return false;
    uint64_t yn;
    if (c < nz && g.w > 1) {
        if (cc != 1) return false;
        yn = (uint64_t)r;
    } else {
        if ((c - 1) % (uint64_t)g.w != 0) return false;
        yn = (c - 1) / (uint64_t)g.w;
        if (yn >= (uint64_t)g.h) return false;
    }
    const int32_t t = nltree_query(fb.nltree, g.nl_size, (int)yn);
    if (t < 0) return false;
    out = Cand{(uint32_t)t, (int32_t)yn, INT_MAX, (uint32_t)'\n'};
    return true;
}

__device__ __forceinline__ Cand shfl_up_cand(const Cand &c)
{
    return Cand{__shfl_up_sync(0xffffffffu, c.tri, 1), __shfl_up_sync(0xffffffffu, c.y, 1),
                __shfl_up_sync(0xffffffffu, c.x, 1), __shfl_up_sync(0xffffffffu, c.cell, 1)};
}

// Resolve frame cells c0 = 2p and c0+1, and depth cells c0 and c0+1, of one frame (the
// rule of resolve_cell).  Called by all 32 lanes of a warp with consecutive p in lane
// order; lanes with valid false (past the end) write nothing.  Depth cell c0-1's winner
// is the previous lane's second depth cell (lane 0 decodes it itself), so a pair costs
// two key reads and two record decodes.
__device__ __forceinline__ void resolve_pair(const FrameGeom &g, const FrameBuffers &fb, uint64_t p, bool valid,
                                             int lane)
{
    const uint64_t nz = (uint64_t)g.w * g.h;
    const uint64_t ncells = g.image ? nz + g.h : nz;
    const uint64_t c0 = 2 * p;
    int r0 = 0, cc0 = 0;
    if (valid && c0 < nz) {
        if (nz <= 0xffffffffull) {
            r0 = (int)((uint32_t)c0 / (uint32_t)g.w);
        } else {
            r0 = (int)(c0 / (uint64_t)g.w);
        }
        cc0 = (int)(c0 - (uint64_t)r0 * g.w);
    }
    int r1 = r0, cc1 = cc0 + 1;
    if (cc1 == g.w) {
        ++r1;
        cc1 = 0;
    }
    Cand k0{0, 0, 0, (uint32_t)' '}, k1{0, 0, 0, (uint32_t)' '};
    bool h0 = false, h1 = false;
    float z0 = kFltMax, z1 = kFltMax;
    if (valid && c0 < nz) {
        const uint64_t k = key_at(g, fb, r0, cc0);
        if (k != kEmptyKey) {
            k0 = decode(g, fb, k, r0, cc0, &z0);
            h0 = true;
        }
    }
    if (valid && c0 + 1 < nz) {
        const uint64_t k = key_at(g, fb, r1, cc1);
        if (k != kEmptyKey) {
            k1 = decode(g, fb, k, r1, cc1, &z1);
            h1 = true;
        }
    }
    // depth cell c0-1
    Cand km = shfl_up_cand(k1);
    bool hm = __shfl_up_sync(0xffffffffu, (int)h1, 1) != 0;
    if (lane == 0) {
        hm = false;
        if (valid && c0 >= 1 && c0 - 1 < nz) {
            int rm, cm;
            if (c0 < nz) {
                rm = cc0 > 0 ? r0 : r0 - 1;
                cm = cc0 > 0 ? cc0 - 1 : g.w - 1;
            } else {
                rm = g.h - 1;
                cm = g.w - 1;
            }
            const uint64_t k = key_at(g, fb, rm, cm);
            if (k != kEmptyKey) {
                km = decode(g, fb, k, rm, cm, nullptr);
                hm = true;
            }
        }
    }
    if (!valid) return;
    // frame cell c0: depth cells c0 and c0-1, newline; frame cell c0+1: c0+1 and c0
    if (c0 < ncells) {
        bool have = h0;
        Cand best = k0;
        if (hm && (!have || later(km, best))) {
            best = km;
            have = true;
        }
        Cand n;
        if (newline_at(g, fb, c0, nz, r0, cc0, n) && (!have || later(n, best))) best = n;
        fb.cells_out[c0] = best.cell;
    }
    if (c0 + 1 < ncells) {
        bool have = h1;
        Cand best = k1;
        if (h0 && (!have || later(k0, best))) {
            best = k0;
            have = true;
        }
        Cand n;
        if (newline_at(g, fb, c0 + 1, nz, r1, cc1, n) && (!have || later(n, best))) best = n;
        fb.cells_out[c0 + 1] = best.cell;
    }
    if (c0 < nz) {
        fb.z_out[c0] = z0;
        fb.winner_out[c0] = h0 ? (int32_t)k0.tri : -1;
    }
    if (c0 + 1 < nz) {
        fb.z_out[c0 + 1] = z1;
        fb.winner_out[c0 + 1] = h1 ? (int32_t)k1.tri : -1;
    }
}

// Resolve frame cells c0 = K*p .. c0+K-1 and the depth cells among them, of one frame
// (the rule of resolve_cell).  Called by all 32 lanes of a warp with consecutive p in
// lane order; lanes with valid false (past the end) write nothing.  Depth cell c0-1's
// winner is the previous lane's last depth cell (lane 0 decodes it itself).  With vec the
// outputs are 4K-byte aligned and a lane's K cells go out in one store per buffer.
template <int K>
__device__ __forceinline__ void resolve_run(const FrameGeom &g, const FrameBuffers &fb, uint64_t p, bool valid,
                                            int lane, bool vec)
{
    static_assert(K == 2 || K == 4, "one 8- or 16-byte store per lane and buffer");
    const uint64_t nz = (uint64_t)g.w * g.h;
    const uint64_t ncells = g.image ? nz + g.h : nz;
    const uint64_t c0 = K * p;
    int r0 = 0, cc0 = 0;
    if (valid && c0 < nz) {
        if (nz <= 0xffffffffull) {
            r0 = (int)((uint32_t)c0 / (uint32_t)g.w);
        } else {
            r0 = (int)(c0 / (uint64_t)g.w);
        }
        cc0 = (int)(c0 - (uint64_t)r0 * g.w);
    }
    int rj[K], cj[K];
    uint64_t key[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        rj[j] = j == 0 ? r0 : (cj[j - 1] + 1 == g.w ? rj[j - 1] + 1 : rj[j - 1]);
        cj[j] = j == 0 ? cc0 : (cj[j - 1] + 1 == g.w ? 0 : cj[j - 1] + 1);
        key[j] = valid && c0 + j < nz ? key_at(g, fb, rj[j], cj[j]) : kEmptyKey;
    }
    Cand kc[K];
    bool hc[K];
    float z[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        kc[j] = Cand{0, 0, 0, (uint32_t)' '};
        hc[j] = key[j] != kEmptyKey;
        z[j] = kFltMax;
        if (hc[j]) kc[j] = decode(g, fb, key[j], rj[j], cj[j], &z[j]);
    }
    // depth cell c0-1
    Cand km = shfl_up_cand(kc[K - 1]);
    bool hm = __shfl_up_sync(0xffffffffu, (int)hc[K - 1], 1) != 0;
    if (lane == 0) {
        hm = false;
        if (valid && c0 >= 1 && c0 - 1 < nz) {
            int rm, cm;
            if (c0 < nz) {
                rm = cc0 > 0 ? r0 : r0 - 1;
                cm = cc0 > 0 ? cc0 - 1 : g.w - 1;
            } else {
                rm = g.h - 1;
                cm = g.w - 1;
            }
            const uint64_t k = key_at(g, fb, rm, cm);
            if (k != kEmptyKey) {
                km = decode(g, fb, k, rm, cm, nullptr);
                hm = true;
            }
        }
    }
    if (!valid) return;
    // frame cell c: depth cells c and c-1, newline
    uint32_t out[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const uint64_t c = c0 + j;
        bool have = hc[j];
        Cand best = kc[j];
        const Cand &prev = j == 0 ? km : kc[j - 1];
        const bool hprev = j == 0 ? hm : hc[j - 1];
        if (hprev && (!have || later(prev, best))) {
            best = prev;
            have = true;
        }
        Cand n;
        if (c < ncells && newline_at(g, fb, c, nz, rj[j], cj[j], n) && (!have || later(n, best))) best = n;
        out[j] = best.cell;
    }
    if (vec && c0 + K <= ncells) {
        if constexpr (K == 4)
            *reinterpret_cast<uint4 *>(fb.cells_out + c0) = make_uint4(out[0], out[1], out[2], out[3]);
        else
            *reinterpret_cast<uint2 *>(fb.cells_out + c0) = make_uint2(out[0], out[1]);
    } else {
#pragma unroll
        for (int j = 0; j < K; ++j)
            if (c0 + j < ncells) fb.cells_out[c0 + j] = out[j];
    }
    if (vec && c0 + K <= nz) {
        int32_t wv[K];
#pragma unroll
        for (int j = 0; j < K; ++j) wv[j] = hc[j] ? (int32_t)kc[j].tri : -1;
        if constexpr (K == 4) {
            *reinterpret_cast<float4 *>(fb.z_out + c0) = make_float4(z[0], z[1], z[2], z[3]);
            *reinterpret_cast<int4 *>(fb.winner_out + c0) = make_int4(wv[0], wv[1], wv[2], wv[3]);
        } else {
            *reinterpret_cast<float2 *>(fb.z_out + c0) = make_float2(z[0], z[1]);
            *reinterpret_cast<int2 *>(fb.winner_out + c0) = make_int2(wv[0], wv[1]);
        }
    } else {
#pragma unroll
        for (int j = 0; j < K; ++j)
            if (c0 + j < nz) {
                fb.z_out[c0 + j] = z[j];
                fb.winner_out[c0 + j] = hc[j] ? (int32_t)kc[j].tri : -1;
            }
    }
}

// Resolve of an even-width frame, pairs of frame cells (c0 = 2p, c0+1).  Samples write
// only even depth columns there (y*w + 2x is even), so depth cell c0+1 never has a winner:
// frame cell c0 takes the winner of depth cell c0 (its left neighbour c0-1 is odd and the
// newline cells y*w+1 are odd), and frame cell c0+1 the later of that winner and, when c0
// starts a row, the row's newline (the rule of resolve_cell).  A thread resolves the J
// pairs p0 + j*stride below pend, issuing every key load first, then every winner's record
// loads, then the arithmetic and stores: J independent chains in flight instead of one.
// With vec the outputs are 8-byte aligned and a pair goes out in one store per buffer.
template <int J>
__device__ __forceinline__ void resolve_even(const FrameGeom &g, const FrameBuffers &fb, uint64_t p0, uint32_t stride,
                                             uint64_t pend, bool vec)
{
    const uint64_t nz = (uint64_t)g.w * g.h;
    const uint64_t ncells = g.image ? nz + g.h : nz;
    uint64_t key[J];
    int rr[J], cc[J];
#pragma unroll
    for (int j = 0; j < J; ++j) {
        const uint64_t c0 = 2 * (p0 + (uint64_t)j * stride);
        key[j] = kEmptyKey;
        rr[j] = 0;
        cc[j] = 0;
        if (c0 < nz) {
            rr[j] = nz <= 0xffffffffull ? (int)((uint32_t)c0 / (uint32_t)g.w) : (int)(c0 / (uint64_t)g.w);
            cc[j] = (int)(c0 - (uint64_t)rr[j] * g.w);
            key[j] = key_at(g, fb, rr[j], cc[j]);
        }
    }
    float4 q0[J], q1[J];
#pragma unroll
    for (int j = 0; j < J; ++j) {
        q0[j] = q1[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (key[j] != kEmptyKey) {
            const float4 *rp = reinterpret_cast<const float4 *>(fb.records + ((uint32_t)key[j] >> 1));
            q0[j] = __ldg(rp);
            q1[j] = __ldg(rp + 1);
        }
    }
#pragma unroll
    for (int j = 0; j < J; ++j) {
        const uint64_t p = p0 + (uint64_t)j * stride;
        if (p >= pend) continue;
        const uint64_t c0 = 2 * p;
        const bool have = key[j] != kEmptyKey;
        float z = kFltMax;
        Cand best{0, 0, 0, (uint32_t)' '};
        if (have) best = decode_rows(g, fb, key[j], rr[j], cc[j], q0[j], q1[j], &z);
        const uint32_t out0 = best.cell;
        // frame cell c0+1: depth cell c0's winner, or the newline of row rr when c0 starts it
        uint32_t out1 = best.cell;
        if (g.image && c0 < nz && cc[j] == 0) {
            const int32_t t = nltree_query(fb.nltree, g.nl_size, rr[j]);
            if (t >= 0) {
                const Cand n{(uint32_t)t, rr[j], INT_MAX, (uint32_t)'\n'};
                if (!have || later(n, best)) out1 = n.cell;
            }
        }
        if (vec && c0 + 2 <= ncells) {
            *reinterpret_cast<uint2 *>(fb.cells_out + c0) = make_uint2(out0, out1);
        } else {
            fb.cells_out[c0] = out0;
            if (c0 + 1 < ncells) fb.cells_out[c0 + 1] = out1;
        }
        if (c0 < nz) {   // nz is even: c0 + 1 < nz too
            const int32_t w0 = have ? (int32_t)best.tri : -1;
            if (vec) {
                *reinterpret_cast<float2 *>(fb.z_out + c0) = make_float2(z, kFltMax);
                *reinterpret_cast<int2 *>(fb.winner_out + c0) = make_int2(w0, -1);
            } else {
                fb.z_out[c0] = z;
                fb.z_out[c0 + 1] = kFltMax;
                fb.winner_out[c0] = w0;
                fb.winner_out[c0 + 1] = -1;
            }
        }
    }
}

}  // namespace sloth
