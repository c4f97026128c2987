// tile_ops.cuh -- device building blocks of the tiled push: field gather from a staged tile,
// per-segment current values, and the warp-cooperative shared-memory current accumulation.
#pragma once

#include "pic_math.cuh"

namespace osg {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Staggered gather from a shared-memory tile of E (or B) stored as [z][y][x][3].
// lf = local point of the particle's cell in the stencil frame, lh = lf - (x < 0).
// E1 (h,f,f) E2 (f,h,f) E3 (f,f,h); B1 (f,h,h) B2 (h,f,h) B3 (h,h,f)  (2D: drop the z entry)
template <int DIM, int ORD>
__device__ __forceinline__ void gather_tile(const float *sE, const float *sB, int esy, int esz,
                                            const int *lf, const int *lh,
                                            const float (*w)[ORD + 1],
                                            const float (*wh)[ORD + 1], float &E1, float &E2,
                                            float &E3, float &B1, float &B2, float &B3)
{
    constexpr int NP = ORD + 1;
    E1 = E2 = E3 = B1 = B2 = B3 = 0.f;
    if constexpr (DIM == 2) {
#pragma unroll
        for (int k2 = 0; k2 < NP; k2++) {
            float f1 = 0.f, f2 = 0.f, f3 = 0.f;
#pragma unroll
            for (int k1 = 0; k1 < NP; k1++) {
                f1 = fmaf(sE[3 * (lh[0] + k1) + esy * (lf[1] + k2) + 0], wh[0][k1], f1);
                f2 = fmaf(sE[3 * (lf[0] + k1) + esy * (lh[1] + k2) + 1], w[0][k1], f2);
                f3 = fmaf(sE[3 * (lf[0] + k1) + esy * (lf[1] + k2) + 2], w[0][k1], f3);
            }
            E1 = fmaf(f1, w[1][k2], E1);
            E2 = fmaf(f2, wh[1][k2], E2);
            E3 = fmaf(f3, w[1][k2], E3);
        }
#pragma unroll
        for (int k2 = 0; k2 < NP; k2++) {
            float f1 = 0.f, f2 = 0.f, f3 = 0.f;
#pragma unroll
            for (int k1 = 0; k1 < NP; k1++) {
                f1 = fmaf(sB[3 * (lf[0] + k1) + esy * (lh[1] + k2) + 0], w[0][k1], f1);
                f2 = fmaf(sB[3 * (lh[0] + k1) + esy * (lf[1] + k2) + 1], wh[0][k1], f2);
                f3 = fmaf(sB[3 * (lh[0] + k1) + esy * (lh[1] + k2) + 2], wh[0][k1], f3);
            }
            B1 = fmaf(f1, wh[1][k2], B1);
            B2 = fmaf(f2, w[1][k2], B2);
            B3 = fmaf(f3, wh[1][k2], B3);
        }
    } else {
#pragma unroll
        for (int k3 = 0; k3 < NP; k3++) {
            float g1 = 0.f, g2 = 0.f, g3 = 0.f;
#pragma unroll
            for (int k2 = 0; k2 < NP; k2++) {
                float f1 = 0.f, f2 = 0.f, f3 = 0.f;
#pragma unroll
                for (int k1 = 0; k1 < NP; k1++) {
                    f1 = fmaf(sE[3 * (lh[0] + k1) + esy * (lf[1] + k2) + esz * (lf[2] + k3) + 0], wh[0][k1], f1);
                    f2 = fmaf(sE[3 * (lf[0] + k1) + esy * (lh[1] + k2) + esz * (lf[2] + k3) + 1], w[0][k1], f2);
                    f3 = fmaf(sE[3 * (lf[0] + k1) + esy * (lf[1] + k2) + esz * (lh[2] + k3) + 2], w[0][k1], f3);
                }
                g1 = fmaf(f1, w[1][k2], g1);
                g2 = fmaf(f2, wh[1][k2], g2);
                g3 = fmaf(f3, w[1][k2], g3);
            }
            E1 = fmaf(g1, w[2][k3], E1);
            E2 = fmaf(g2, w[2][k3], E2);
            E3 = fmaf(g3, wh[2][k3], E3);
        }
#pragma unroll
        for (int k3 = 0; k3 < NP; k3++) {
            float g1 = 0.f, g2 = 0.f, g3 = 0.f;
#pragma unroll
            for (int k2 = 0; k2 < NP; k2++) {
                float f1 = 0.f, f2 = 0.f, f3 = 0.f;
#pragma unroll
                for (int k1 = 0; k1 < NP; k1++) {
                    f1 = fmaf(sB[3 * (lf[0] + k1) + esy * (lh[1] + k2) + esz * (lh[2] + k3) + 0], w[0][k1], f1);
                    f2 = fmaf(sB[3 * (lh[0] + k1) + esy * (lf[1] + k2) + esz * (lh[2] + k3) + 1], wh[0][k1], f2);
                    f3 = fmaf(sB[3 * (lh[0] + k1) + esy * (lh[1] + k2) + esz * (lf[2] + k3) + 2], wh[0][k1], f3);
                }
                g1 = fmaf(f1, wh[1][k2], g1);
                g2 = fmaf(f2, w[1][k2], g2);
                g3 = fmaf(f3, wh[1][k2], g3);
            }
            B1 = fmaf(g1, wh[2][k3], B1);
            B2 = fmaf(g2, wh[2][k3], B2);
            B3 = fmaf(g3, w[2][k3], B3);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Current values of one segment, in a fixed order; seg_offset maps a value index to its
// offset (in floats) from the stencil origin of the segment's cell in the shared tile.
//   2D: j1 [k2 < NP][k1 < ORD], j2 [k2 < ORD][k1 < NP], j3 [k2 < NP][k1 < NP]
//   3D: j1 [k3][k2][k1 < ORD],  j2 [k3][k2 < ORD][k1],  j3 [k3 < ORD][k2][k1]
// ------------------------------------------------------------------------------------------
template <int DIM, int ORD> struct SegVals {
    static constexpr int NP = ORD + 1;
    static constexpr int NV = DIM == 2 ? 2 * ORD * NP + NP * NP : 3 * ORD * NP * NP;
};

template <int ORD>
__device__ __forceinline__ void seg_values2(const Seg2<float> &g, float q, float jn0, float jn1,
                                            float *v)
{
    constexpr int NP = ORD + 1;
    float s0x[NP], s1x[NP], s0y[NP], s1y[NP], wl1[ORD], wl2[ORD];
    spline<ORD>(g.x0, s0x);
    spline<ORD>(g.x1, s1x);
    spline<ORD>(g.y0, s0y);
    spline<ORD>(g.y1, s1y);
    const float qvz = (q * g.vz) * float(1.0 / 3.0);
    long_weights<ORD>(q * jn0, g.x0, g.x1, wl1);
    long_weights<ORD>(q * jn1, g.y0, g.y1, wl2);
    int n = 0;
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++) {
        const float wp1 = s0y[k2] + s1y[k2];
#pragma unroll
        for (int k1 = 0; k1 < ORD; k1++) v[n++] = wl1[k1] * wp1;
    }
#pragma unroll
    for (int k2 = 0; k2 < ORD; k2++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) v[n++] = wl2[k2] * (s0x[k1] + s1x[k1]);
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            float t1 = fmaf(s1y[k2], s1x[k1], s0x[k1] * s0y[k2]);
            const float t2 = fmaf(s0y[k2], s1x[k1], s0x[k1] * s1y[k2]);
            t1 = fmaf(t2, 0.5f, t1);
            v[n++] = qvz * t1;
        }
}

template <int ORD>
__device__ __forceinline__ void seg_values3(const Seg3<float> &g, float q, const float *jn,
                                            float *v)
{
    constexpr int NP = ORD + 1;
    float s0x[NP], s1x[NP], s0y[NP], s1y[NP], s0z[NP], s1z[NP];
    float wl1[ORD], wl2[ORD], wl3[ORD];
    spline<ORD>(g.x0, s0x);
    spline<ORD>(g.x1, s1x);
    spline<ORD>(g.y0, s0y);
    spline<ORD>(g.y1, s1y);
    spline<ORD>(g.z0, s0z);
    spline<ORD>(g.z1, s1z);
    long_weights<ORD>(q * jn[0], g.x0, g.x1, wl1);
    long_weights<ORD>(q * jn[1], g.y0, g.y1, wl2);
    long_weights<ORD>(q * jn[2], g.z0, g.z1, wl3);
    int n = 0;
#pragma unroll
    for (int k3 = 0; k3 < NP; k3++)
#pragma unroll
        for (int k2 = 0; k2 < NP; k2++) {
            float t1 = s0y[k2] * s0z[k3], t2 = s0y[k2] * s1z[k3];
            t1 = fmaf(s1y[k2], s1z[k3], t1);
            t2 = fmaf(s1y[k2], s0z[k3], t2);
            const float wp = fmaf(0.5f, t2, t1);
#pragma unroll
            for (int k1 = 0; k1 < ORD; k1++) v[n++] = wl1[k1] * wp;
        }
#pragma unroll
    for (int k3 = 0; k3 < NP; k3++)
#pragma unroll
        for (int k2 = 0; k2 < ORD; k2++)
#pragma unroll
            for (int k1 = 0; k1 < NP; k1++) {
                float t1 = s0x[k1] * s0z[k3], t2 = s0x[k1] * s1z[k3];
                t1 = fmaf(s1x[k1], s1z[k3], t1);
                t2 = fmaf(s1x[k1], s0z[k3], t2);
                v[n++] = wl2[k2] * fmaf(0.5f, t2, t1);
            }
#pragma unroll
    for (int k3 = 0; k3 < ORD; k3++)
#pragma unroll
        for (int k2 = 0; k2 < NP; k2++)
#pragma unroll
            for (int k1 = 0; k1 < NP; k1++) {
                float t1 = s0x[k1] * s0y[k2], t2 = s0x[k1] * s1y[k2];
                t1 = fmaf(s1x[k1], s1y[k2], t1);
                t2 = fmaf(s1x[k1], s0y[k2], t2);
                v[n++] = wl3[k3] * fmaf(0.5f, t2, t1);
            }
}

// direct shared-memory accumulation of one 3D segment (pj = stencil origin)
template <int ORD>
__device__ __forceinline__ void seg_atomic3(float *pj, const Seg3<float> &g, float q,
                                            const float *jn, int jsy, int jsz)
{
    constexpr int NP = ORD + 1;
    float s0x[NP], s1x[NP], s0y[NP], s1y[NP], s0z[NP], s1z[NP];
    float wl1[ORD], wl2[ORD], wl3[ORD];
    spline<ORD>(g.x0, s0x);
    spline<ORD>(g.x1, s1x);
    spline<ORD>(g.y0, s0y);
    spline<ORD>(g.y1, s1y);
    spline<ORD>(g.z0, s0z);
    spline<ORD>(g.z1, s1z);
    long_weights<ORD>(q * jn[0], g.x0, g.x1, wl1);
    long_weights<ORD>(q * jn[1], g.y0, g.y1, wl2);
    long_weights<ORD>(q * jn[2], g.z0, g.z1, wl3);
#pragma unroll
    for (int k3 = 0; k3 < NP; k3++)
#pragma unroll
        for (int k2 = 0; k2 < NP; k2++) {
            float t1 = s0y[k2] * s0z[k3], t2 = s0y[k2] * s1z[k3];
            t1 = fmaf(s1y[k2], s1z[k3], t1);
            t2 = fmaf(s1y[k2], s0z[k3], t2);
            const float wp = fmaf(0.5f, t2, t1);
#pragma unroll
            for (int k1 = 0; k1 < ORD; k1++) atomicAdd(pj + 3 * k1 + jsy * k2 + jsz * k3, wl1[k1] * wp);
        }
#pragma unroll
    for (int k3 = 0; k3 < NP; k3++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            float t1 = s0x[k1] * s0z[k3], t2 = s0x[k1] * s1z[k3];
            t1 = fmaf(s1x[k1], s1z[k3], t1);
            t2 = fmaf(s1x[k1], s0z[k3], t2);
            const float wp = fmaf(0.5f, t2, t1);
#pragma unroll
            for (int k2 = 0; k2 < ORD; k2++)
                atomicAdd(pj + 3 * k1 + jsy * k2 + jsz * k3 + 1, wl2[k2] * wp);
        }
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            float t1 = s0x[k1] * s0y[k2], t2 = s0x[k1] * s1y[k2];
            t1 = fmaf(s1x[k1], s1y[k2], t1);
            t2 = fmaf(s1x[k1], s0y[k2], t2);
            const float wp = fmaf(0.5f, t2, t1);
#pragma unroll
            for (int k3 = 0; k3 < ORD; k3++)
                atomicAdd(pj + 3 * k1 + jsy * k2 + jsz * k3 + 2, wl3[k3] * wp);
        }
}

template <int DIM, int ORD>
__device__ __forceinline__ int seg_offset(int vi, int jsy, int jsz)
{
    constexpr int NP = ORD + 1;
    if constexpr (DIM == 2) {
        if (vi < ORD * NP) return 3 * (vi % ORD) + jsy * (vi / ORD);
        vi -= ORD * NP;
        if (vi < ORD * NP) return 3 * (vi % NP) + jsy * (vi / NP) + 1;
        vi -= ORD * NP;
        return 3 * (vi % NP) + jsy * (vi / NP) + 2;
    } else {
        constexpr int B = ORD * NP * NP;
        if (vi < B) return 3 * (vi % ORD) + jsy * ((vi / ORD) % NP) + jsz * (vi / (ORD * NP));
        vi -= B;
        if (vi < B) return 3 * (vi % NP) + jsy * ((vi / NP) % ORD) + jsz * (vi / (ORD * NP)) + 1;
        vi -= B;
        return 3 * (vi % NP) + jsy * ((vi / NP) % NP) + jsz * (vi / (NP * NP)) + 2;
    }
}

// Reduce 32 values held by every lane across the warp so that lane l ends with the warp sum
// of value l (recursive halving: 31 shuffles for 32 sums).
__device__ __forceinline__ float transpose_reduce32(float (&t)[32])
{
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const bool upper = (lane & step) != 0;
#pragma unroll
        for (int k = 0; k < step; k++) {
            const float send = upper ? t[k] : t[k + step];
            const float keep = upper ? t[k + step] : t[k];
            t[k] = keep + __shfl_xor_sync(FULL_MASK, send, step);
        }
    }
    return t[0];
}

// Warp-cooperative accumulation of one segment per lane into the shared current tile.
// base = offset of the lane's stencil origin, or -1 when the lane has no segment.  Lanes whose
// cell is shared by at least `reduce_min` lanes of the warp are summed in registers first
// (transpose-reduce, one pass per such cell), so every shared-memory add of a pass hits a
// distinct address and lanes that deposit into the same cell never serialise on conflicting
// atomics.  Lanes of sparsely populated cells (fewer peers) add their values directly: a
// reduce pass costs about four times a direct pass, which only pays when many lanes share it.
template <int DIM, int ORD>
__device__ __forceinline__ void warp_deposit(float *sJ, int base, const float *v, int jsy,
                                             int jsz, int reduce_min)
{
    constexpr int NV = SegVals<DIM, ORD>::NV;
    constexpr int NB = (NV + 31) / 32;
    const unsigned lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(FULL_MASK, base);
    const bool active = base >= 0;
    const bool direct = active && __popc(peers) < reduce_min;
    if (direct) {
#pragma unroll
        for (int i = 0; i < NV; i++) atomicAdd(sJ + base + seg_offset<DIM, ORD>(i, jsy, jsz), v[i]);
    }
    unsigned rem = __ballot_sync(FULL_MASK, active && !direct && (__ffs(peers) - 1) == (int)lane);
    while (rem) {
        const int l = __ffs(rem) - 1;
        rem &= rem - 1;
        const int key = __shfl_sync(FULL_MASK, base, l);
        const bool mine = base == key;
#pragma unroll
        for (int bch = 0; bch < NB; bch++) {
            float t[32];
#pragma unroll
            for (int k = 0; k < 32; k++) {
                const int i = bch * 32 + k;
                t[k] = (i < NV && mine) ? v[i < NV ? i : 0] : 0.f;
            }
            const float sum = transpose_reduce32(t);
            const int i = bch * 32 + (int)lane;
            if (i < NV) atomicAdd(sJ + key + seg_offset<DIM, ORD>(i, jsy, jsz), sum);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Segment records in the shared segment buffer: a = {x0, x1, y0, y1, z0, z1} (2D: a[4] = vz),
// base = offset of the segment's stencil origin in the shared current tile (-1 = empty).
// ------------------------------------------------------------------------------------------
struct alignas(16) SegRec {
    float a[6];
    float q;
    int base;
};

template <int DIM>
__device__ __forceinline__ int make_segments(SegRec *out, const float *xo, const float *x1,
                                             const int *di, float vz, float q, int li, int lj,
                                             int lk, int jsy, int jsz)
{
    if constexpr (DIM == 2) {
        Seg2<float> sg[3];
        sg[0].x0 = xo[0]; sg[0].x1 = x1[0]; sg[0].y0 = xo[1]; sg[0].y1 = x1[1];
        sg[0].vz = vz; sg[0].i = li; sg[0].j = lj;
        const int n = split2(sg, di[0], di[1]);
#pragma unroll
        for (int t = 0; t < 3; t++) {
            out[t].a[0] = sg[t].x0; out[t].a[1] = sg[t].x1;
            out[t].a[2] = sg[t].y0; out[t].a[3] = sg[t].y1;
            out[t].a[4] = sg[t].vz; out[t].a[5] = 0.f;
            out[t].q = q;
            out[t].base = 3 * sg[t].i + jsy * sg[t].j;
        }
        return n;
    } else {
        Seg3<float> sg[4];
        sg[0].x0 = xo[0]; sg[0].x1 = x1[0]; sg[0].y0 = xo[1]; sg[0].y1 = x1[1];
        sg[0].z0 = xo[2]; sg[0].z1 = x1[2];
        sg[0].i = li; sg[0].j = lj; sg[0].k = lk;
        const int n = split3(sg, di[0], di[1], di[2]);
#pragma unroll
        for (int t = 0; t < 4; t++) {
            out[t].a[0] = sg[t].x0; out[t].a[1] = sg[t].x1;
            out[t].a[2] = sg[t].y0; out[t].a[3] = sg[t].y1;
            out[t].a[4] = sg[t].z0; out[t].a[5] = sg[t].z1;
            out[t].q = q;
            out[t].base = 3 * sg[t].i + jsy * sg[t].j + jsz * sg[t].k;
        }
        return n;
    }
}

// lane order that puts the particles of one warp nthr/32 slots apart (consecutive particles
// usually share a cell; spreading them removes most shared-memory address conflicts)
__device__ __forceinline__ int spread_index(int t, int nthr)
{
    return (t & 31) * (nthr >> 5) + (t >> 5);
}

// Deposit one segment per lane (rec = nullptr: no segment).  reduce_min > 32 selects plain
// per-lane shared atomics (no warp-synchronous part); otherwise warp_deposit.  3D cubic and
// quartic segments (144 and 300 values) always add directly: their values do not fit in
// registers next to a reduce buffer.
template <int DIM, int ORD>
constexpr bool direct_only() { return DIM == 3 && ORD >= 3; }

template <int DIM, int ORD>
__device__ __forceinline__ void deposit_segment(float *sJ, const SegRec *rec, const float *jn,
                                                int jsy, int jsz, int reduce_min)
{
    if constexpr (DIM == 3) {
        if (direct_only<DIM, ORD>() || reduce_min > 32) {
            if (rec) {
                Seg3<float> g;
                g.x0 = rec->a[0]; g.x1 = rec->a[1]; g.y0 = rec->a[2]; g.y1 = rec->a[3];
                g.z0 = rec->a[4]; g.z1 = rec->a[5]; g.i = g.j = g.k = 0;
                seg_atomic3<ORD>(sJ + rec->base, g, rec->q, jn, jsy, jsz);
            }
            return;
        }
    }
    if constexpr (!direct_only<DIM, ORD>()) {
    constexpr int NV = SegVals<DIM, ORD>::NV;
    float v[NV];
    int base = -1;
    if (rec) {
        if constexpr (DIM == 2) {
            Seg2<float> g;
            g.x0 = rec->a[0]; g.x1 = rec->a[1]; g.y0 = rec->a[2]; g.y1 = rec->a[3];
            g.vz = rec->a[4]; g.i = 0; g.j = 0;
            seg_values2<ORD>(g, rec->q, jn[0], jn[1], v);
        } else {
            Seg3<float> g;
            g.x0 = rec->a[0]; g.x1 = rec->a[1]; g.y0 = rec->a[2]; g.y1 = rec->a[3];
            g.z0 = rec->a[4]; g.z1 = rec->a[5]; g.i = g.j = g.k = 0;
            seg_values3<ORD>(g, rec->q, jn, v);
        }
        base = rec->base;
    } else {
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = 0.f;
    }
    warp_deposit<DIM, ORD>(sJ, base, v, jsy, jsz, reduce_min);
    }
}

} // namespace osg
