// tile_ops.cuh -- device building blocks of the tiled push: field gather from a staged tile,
// per-segment current values, and the warp-cooperative shared-memory current accumulation.
#pragma once

#include <climits>

#include "pic_math.cuh"

namespace osg {

constexpr unsigned FULL_MASK = 0xffffffffu;

// *hi += v, with the rounding error of the addition accumulated in *lo (two-sum: the pair
// hi + lo keeps the sum of all added values to about twice the float precision).  Plain
// read-modify-write: the caller owns the address (a warp-private current tile, no other lane
// of the same instruction on it).
__device__ __forceinline__ void comp_add(float *hi, float *lo, float v)
{
    const float a = *hi, t = a + v;
    const float bv = t - a;
    const float err = (a - (t - bv)) + (v - bv);
    *hi = t;
    *lo += err;
}

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

// 2D gather with paired FP32 FMAs (sm_100+ FFMA2: two independent IEEE fmas per instruction):
// the six components share their stencils in pairs -- (E1, B2) weights (wh, w) in (x, y) and
// the same points, (E2, B1) weights (w, wh) and the same points, (E3, B3) -- so every pair is
// one paired fma per stencil point.  Same roundings as gather_tile.
template <int ORD>
__device__ __forceinline__ void gather_tile2_paired(const float *sE, const float *sB, int esy,
                                                    const int *lf, const int *lh,
                                                    const float (*w)[ORD + 1],
                                                    const float (*wh)[ORD + 1], float &E1,
                                                    float &E2, float &E3, float &B1, float &B2,
                                                    float &B3)
{
    constexpr int NP = ORD + 1;
    float2 eb12 = make_float2(0.f, 0.f);   // (E1, B2)
    float2 eb21 = make_float2(0.f, 0.f);   // (E2, B1)
    float2 eb33 = make_float2(0.f, 0.f);   // (E3, B3)
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++) {
        float2 f12 = make_float2(0.f, 0.f), f21 = make_float2(0.f, 0.f), f33 = make_float2(0.f, 0.f);
        const int rf = esy * (lf[1] + k2), rh = esy * (lh[1] + k2);
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            const int xh = 3 * (lh[0] + k1), xf = 3 * (lf[0] + k1);
            f12 = __ffma2_rn(make_float2(sE[xh + rf + 0], sB[xh + rf + 1]),
                             make_float2(wh[0][k1], wh[0][k1]), f12);
            f21 = __ffma2_rn(make_float2(sE[xf + rh + 1], sB[xf + rh + 0]),
                             make_float2(w[0][k1], w[0][k1]), f21);
            f33 = __ffma2_rn(make_float2(sE[xf + rf + 2], sB[xh + rh + 2]),
                             make_float2(w[0][k1], wh[0][k1]), f33);
        }
        eb12 = __ffma2_rn(f12, make_float2(w[1][k2], w[1][k2]), eb12);
        eb21 = __ffma2_rn(f21, make_float2(wh[1][k2], wh[1][k2]), eb21);
        eb33 = __ffma2_rn(f33, make_float2(w[1][k2], wh[1][k2]), eb33);
    }
    E1 = eb12.x; B2 = eb12.y;
    E2 = eb21.x; B1 = eb21.y;
    E3 = eb33.x; B3 = eb33.y;
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

template <int ORD, typename T = float>
__device__ __forceinline__ void seg_values2(const Seg2<T> &g, T q, T jn0, T jn1, T *v)
{
    constexpr int NP = ORD + 1;
    T s0x[NP], s1x[NP], s0y[NP], s1y[NP], wl1[ORD], wl2[ORD];
    spline<ORD>(g.x0, s0x);
    spline<ORD>(g.x1, s1x);
    spline<ORD>(g.y0, s0y);
    spline<ORD>(g.y1, s1y);
    const T qvz = (q * g.vz) * T(1.0 / 3.0);
    long_weights<ORD>(q * jn0, g.x0, g.x1, wl1);
    long_weights<ORD>(q * jn1, g.y0, g.y1, wl2);
    int n = 0;
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++) {
        const T wp1 = s0y[k2] + s1y[k2];
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
            T t1 = fmaR(s1y[k2], s1x[k1], s0x[k1] * s0y[k2]);
            const T t2 = fmaR(s0y[k2], s1x[k1], s0x[k1] * s1y[k2]);
            t1 = fmaR(t2, T(0.5), t1);
            v[n++] = qvz * t1;
        }
}

// The same values for the mixed-precision (tiled) engine with fewer operations: the j3 term
// qvz (s0x s0y + s1x s1y + (s0x s1y + s1x s0y) / 2) is factored as s0x A + s1x B with
// A = qvz (s0y + s1y / 2), B = qvz (s1y + s0y / 2) (two operations per value instead of six;
// the roundings differ from the reference's order by a few float ulps).
template <int ORD>
__device__ __forceinline__ void seg_values2_fast(const Seg2<float> &g, float q, float jn0,
                                                 float jn1, float *v)
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
    for (int k2 = 0; k2 < NP; k2++) {
        const float A = qvz * fmaf(0.5f, s1y[k2], s0y[k2]);
        const float B = qvz * fmaf(0.5f, s0y[k2], s1y[k2]);
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) v[n++] = fmaf(s1x[k1], B, s0x[k1] * A);
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

// ------------------------------------------------------------------------------------------
// Segment record (held in registers): a = {x0, x1, y0, y1, z0, z1} (2D: a[4] = vz),
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

// ------------------------------------------------------------------------------------------
// 2D deposit through a per-warp scratch of segment values.  Every warp of the push CTA owns a
// copy of the current tile (hi, with a two-sum compensation lo at offset jlo), so every add
// below is a plain shared read-modify-write: no lane of the same instruction shares an address
// (shared-memory FP32 atomics are compare-and-swap loops on this GPU).  Lanes write the NV
// values of their segment as rows of the scratch (column-major: value k of row r at
// k * SCR_LD + r, the row's stencil origin in a last column), 16 rows at a time; then lane k
// sums column k.  The in-cell segments of a cell-sorted tile form runs of consecutive rows
// with one stencil origin: lane k adds each run's sum once, so a warp pays one column pass
// whatever the number of cells it covers.  Face-crossing segments (scattered, few) wait in a
// per-warp queue and are added row by row, 32 at a time.
// ------------------------------------------------------------------------------------------
constexpr int SCR_ROWS = 16;
constexpr int SCR_LD = 20;   // column stride: 16-byte aligned, 5 16-byte units (bank spread)

// floats of one warp's scratch (NV value columns and the stencil-origin column)
template <int ORD>
constexpr int scratch_floats2() { return (SegVals<2, ORD>::NV + 1) * SCR_LD; }

// offsets (from a stencil origin) of the columns this lane sums: lane, lane + 32, ...
template <int ORD> struct ColSlots {
    static constexpr int NV = SegVals<2, ORD>::NV;
    static constexpr int NC = (NV + 31) / 32;
    int off[NC];
    __device__ __forceinline__ void init(int jsy)
    {
        const int lane = (int)(threadIdx.x & 31);
#pragma unroll
        for (int c = 0; c < NC; c++)
            off[c] = lane + 32 * c < NV ? seg_offset<2, ORD>(lane + 32 * c, jsy, 0) : 0;
    }
};

// lanes 16 h .. 16 h + 15 write their values and stencil origin as rows 0..15
template <int ORD>
__device__ __forceinline__ void scratch_half2(float *scr, int h, int base, const float *v)
{
    constexpr int NV = SegVals<2, ORD>::NV;
    const int lane = (int)(threadIdx.x & 31);
    if ((lane >> 4) == h) {
        const int r = lane & 15;
#pragma unroll
        for (int k = 0; k < NV; k++) scr[k * SCR_LD + r] = v[k];
        reinterpret_cast<int *>(scr + NV * SCR_LD)[r] = base;
    }
}

// In-cell segments of the warp (one per lane; base = stencil origin, -1 = none; v = values):
// runs of equal base in lane order are summed per column and added once per run into the
// warp's current tile.  A half of 16 rows inside one run is summed as a pairwise tree (so a
// run of 2^k equal values sums exactly), rows around a run boundary one by one.  Must be
// called by all 32 lanes.
template <int ORD>
__device__ __forceinline__ void cell_runs_deposit2(float *sJ, int jlo, float *scr, int base,
                                                   const float *v, const ColSlots<ORD> &cs)
{
    constexpr int NV = SegVals<2, ORD>::NV;
    constexpr int NC = ColSlots<ORD>::NC;
    const int lane = (int)(threadIdx.x & 31);
    const int prev = __shfl_up_sync(FULL_MASK, base, 1);
    // bit r (r < 31): row r is the last of its run; row 31 ends the last run
    const unsigned ends = __ballot_sync(FULL_MASK, lane > 0 && prev != base) >> 1;
    const int last = __shfl_sync(FULL_MASK, base, 31);
    const int *sb = reinterpret_cast<const int *>(scr + NV * SCR_LD);
    float acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        scratch_half2<ORD>(scr, h, base, v);
        __syncwarp();
        const unsigned eh = (ends >> (SCR_ROWS * h)) & 0xffffu;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int col = lane + 32 * c;
            if (col < NV) {
                const float *cv = scr + col * SCR_LD;
                const float4 *cv4 = reinterpret_cast<const float4 *>(cv);
                if (eh == 0) {
                    const float4 x0 = cv4[0], x1 = cv4[1], x2 = cv4[2], x3 = cv4[3];
                    const float b0 = (x0.x + x0.y) + (x0.z + x0.w);
                    const float b1 = (x1.x + x1.y) + (x1.z + x1.w);
                    const float b2 = (x2.x + x2.y) + (x2.z + x2.w);
                    const float b3 = (x3.x + x3.y) + (x3.z + x3.w);
                    acc[c] += (b0 + b1) + (b2 + b3);
                } else {
                    float *hj = sJ + cs.off[c];
                    float a = acc[c];
#pragma unroll 1
                    for (int b = 0; b < SCR_ROWS / 4; b++) {
                        const unsigned e = (eh >> (4 * b)) & 0xfu;
                        if (e == 0) {
                            const float4 x = cv4[b];
                            a += (x.x + x.y) + (x.z + x.w);
                        } else {
#pragma unroll 1
                            for (int i = 0; i < 4; i++) {
                                a += cv[4 * b + i];
                                if (e & (1u << i)) {
                                    const int key = sb[4 * b + i];
                                    if (key >= 0) comp_add(hj + key, hj + jlo + key, a);
                                    a = 0.f;
                                }
                            }
                        }
                    }
                    acc[c] = a;
                }
            }
        }
        __syncwarp();
    }
    if (last >= 0) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            float *hj = sJ + cs.off[c] + last;
            if (lane + 32 * c < NV) comp_add(hj, hj + jlo, acc[c]);
        }
    }
}

template <int ORD>
__device__ __forceinline__ Seg2<float> seg2_of(const SegRec &r)
{
    Seg2<float> g;
    g.x0 = r.a[0]; g.x1 = r.a[1]; g.y0 = r.a[2]; g.y1 = r.a[3];
    g.vz = r.a[4]; g.i = 0; g.j = 0;
    return g;
}

// Per-warp queue (shared memory) of 2D face-crossing segments waiting to be deposited by a
// full warp: few per iteration and scattered over the lanes; queued, their values are
// computed 32 at a time with every lane busy.
constexpr int SEGQ = 64;

// append r for every lane with put; qn (warp-uniform) is the queue length
__device__ __forceinline__ void segq_push(SegRec *sq, int &qn, bool put, const SegRec &r)
{
    const unsigned lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(FULL_MASK, put);
    if (put) sq[qn + __popc(m & ((1u << lane) - 1u))] = r;
    qn += __popc(m);
}

// deposit the top 32 entries while at least nmin (>= 1) are queued: values into the scratch,
// then row by row, lane k adding value k of the row (distinct addresses within every add;
// plain FP32 adds: the crossings carry a small part of the current, and compensating them
// measured 2.4% slower).  Inlined: as a call it cost 9% of the push (register saves around
// the call)
template <int ORD>
__device__ __forceinline__ void segq_drain(float *sJ, SegRec *sq, int &qn, int nmin,
                                        const float *jn, float *scr, const ColSlots<ORD> &cs)
{
    constexpr int NV = SegVals<2, ORD>::NV;
    const int lane = (int)(threadIdx.x & 31);
    const int *sb = reinterpret_cast<const int *>(scr + NV * SCR_LD);
    while (qn >= nmin) {
        const int take = qn < 32 ? qn : 32, first = qn - take;
        __syncwarp();
        float v[NV];
        int base = -1;
        if (lane < take) {
            const SegRec r = sq[first + lane];
            seg_values2_fast<ORD>(seg2_of<ORD>(r), r.q, jn[0], jn[1], v);
            base = r.base;
        } else {
#pragma unroll
            for (int i = 0; i < NV; i++) v[i] = 0.f;
        }
        qn = first;
#pragma unroll 1
        for (int h = 0; 16 * h < take; h++) {
            __syncwarp();
            scratch_half2<ORD>(scr, h, base, v);
            __syncwarp();
            const int rows = min(take - 16 * h, 16);
#pragma unroll
            for (int c = 0; c < ColSlots<ORD>::NC; c++) {
                const int col = lane + 32 * c;
                if (col < NV) {
                    const float *cv = scr + col * SCR_LD;
                    float *hj = sJ + cs.off[c];
#pragma unroll 1
                    for (int r = 0; r < rows; r++) hj[sb[r]] += cv[r];
                }
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------------
// 3D deposit.  The CTA's current tile is one shared copy, accumulated exactly as fixed point
// (value x 2^S rounded to an integer, v) in two 32-bit words per point: the high word sums
// v >> B (signed), the low word sums v itself, modulo 2^32.  Both are plain 32-bit integer adds
// with no return value (FP32 shared-memory atomics are compare-and-swap loops on this GPU).  The
// host picks S and B from the most adds a point can take in one step, N, so that the high word
// cannot overflow and N 2^B <= 2^32.  The sum of the low B bits of every v, sum - hi 2^B, then
// lies in [0, 2^32) and equals lo - hi 2^B modulo 2^32: the point's value is
// hi 2^B + (unsigned)(lo - hi 2^B) (k_tile_fold).  The tile sums therefore carry no rounding
// beyond the one of each added value (to a multiple of 2^-S, an absolute quantum) and do not
// depend on the order of the adds.  Every lane adds the values of its own segment
// (lanes_deposit3); the face crossings wait in a per-warp queue so that they are deposited by
// full warps.
// ------------------------------------------------------------------------------------------
constexpr int SEGQ3 = 48;        // queued face crossings per warp
constexpr int SEGQ3_KEEP = 16;   // drain while more than this many wait (a round adds <= 32)

// fixed-point format of the 3D tile current: scale = 2^S, shift = B
struct FxFormat {
    float scale;
    int shift;
};

// add v (a fixed-point value) to the point whose words are lo and hi
__device__ __forceinline__ void fx_add(unsigned *lo, unsigned *hi, int v, int shift)
{
    atomicAdd(lo, (unsigned)v);
    atomicAdd(hi, (unsigned)(v >> shift));
}

// B-spline weights at both ends and longitudinal weights (q jn folded in) of one 3D segment
template <int ORD> struct Seg3W {
    static constexpr int NP = ORD + 1;
    float s0[3][NP], s1[3][NP], wl[3][ORD];
};

template <int ORD>
__device__ __forceinline__ void seg3_weights(const SegRec &r, const float *jn, Seg3W<ORD> &w)
{
#pragma unroll
    for (int d = 0; d < 3; d++) {
        spline<ORD>(r.a[2 * d], w.s0[d]);
        spline<ORD>(r.a[2 * d + 1], w.s1[d]);
        long_weights<ORD>(r.q * jn[d], r.a[2 * d], r.a[2 * d + 1], w.wl[d]);
    }
}

// weight across the motion along axis pair (a, b): s0a s0b + s1a s1b + (s0a s1b + s1a s0b) / 2
// (DEP_CURRENT_3D, source/spec/os-spec-current.f03:2800-2905)
__device__ __forceinline__ float wperp(float s0a, float s1a, float s0b, float s1b)
{
    float t1 = s0a * s0b, t2 = s0a * s1b;
    t1 = fmaf(s1a, s1b, t1);
    t2 = fmaf(s1a, s0b, t2);
    return fmaf(0.5f, t2, t1);
}

// v[k] for a runtime index k < N (a chain of selects: the arrays stay in registers)
template <int N>
__device__ __forceinline__ float pick(const float (&v)[N], int k)
{
    float r = v[0];
#pragma unroll
    for (int j = 1; j < N; j++) r = k == j ? v[j] : r;
    return r;
}

// One 3D segment per lane (has = false: none), each lane adding its own values straight into
// the tile.  The values come in 3 (ORD + 1) blocks of ORD (ORD + 1) -- block (c, k) holds
// component c at plane k: j1 and j2 over z planes, j3 over y planes -- each the outer product
// of the longitudinal weights of c with a perpendicular weight vector.  Lanes of one cell (up
// to 8 or so in a cell-sorted tile) must add to different addresses in each atomic
// instruction:
// - orders >= 2: the components go in a fixed order (their strides and weights known at
//   compile time); within a component a lane starts at plane lane mod (ORD + 1) and at
//   longitudinal index (lane / (ORD + 1)) mod ORD, so lanes of one cell take different
//   (plane, index) pairs -- (ORD + 1) ORD of them;
// - linear (two planes, one index): the lanes rotate over all 6 blocks instead.
// The plane loop is not unrolled (small code; selects pick the plane's weights).
template <int ORD>
__device__ __noinline__ void lanes_deposit3(unsigned *Jl, unsigned *Jh, const SegRec r,
                                            bool has, const float *jn, int jsy, int jsz,
                                            FxFormat fx)
{
    constexpr int NP = ORD + 1, NBLK = 3 * NP;
    if (!has) return;
    Seg3W<ORD> w;
    seg3_weights<ORD>(r, jn, w);
    // the longitudinal weights in fixed-point units (the scale is a power of two: exact)
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int i = 0; i < ORD; i++) w.wl[d][i] *= fx.scale;
    unsigned *jl = Jl + r.base, *jh = Jh + r.base;
    const int lane = (int)(threadIdx.x & 31);
    if constexpr (ORD >= 2) {
        const int rk = lane % NP, ri = (lane / NP) % ORD;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            // perpendicular axes: A (y for j1, x for j2, j3) and B, the plane axis (z for j1,
            // j2; y for j3)
            const int ax = c == 0 ? 1 : 0, bx = c == 2 ? 1 : 2;
            const int si = c == 0 ? 3 : (c == 1 ? jsy : jsz);
            const int sm = c == 0 ? jsy : 3;
            const int sk = c == 2 ? jsy : jsz;
            float a[ORD];
            int ao[ORD];
#pragma unroll
            for (int i = 0; i < ORD; i++) {
                int ii = i + ri;
                if (ii >= ORD) ii -= ORD;
                a[i] = pick(w.wl[c], ii);
                ao[i] = si * ii;
            }
#pragma unroll 1
            for (int t = 0; t < NP; t++) {
                int k = t + rk;
                if (k >= NP) k -= NP;
                const float B0 = pick(w.s0[bx], k), B1 = pick(w.s1[bx], k);
                const int o0 = c + sk * k;
#pragma unroll
                for (int m = 0; m < NP; m++) {
                    const float wp = wperp(w.s0[ax][m], w.s1[ax][m], B0, B1);
#pragma unroll
                    for (int i = 0; i < ORD; i++) {
                        const int o = o0 + ao[i] + sm * m;
                        fx_add(jl + o, jh + o, __float2int_rn(a[i] * wp), fx.shift);
                    }
                }
            }
        }
    } else {
        const int rot = lane % NBLK;
#pragma unroll 1
        for (int t = 0; t < NBLK; t++) {
            int blk = t + rot;
            if (blk >= NBLK) blk -= NBLK;
            const int c = blk / NP, k = blk - c * NP;
            float a[ORD], A0[NP], A1[NP];
#pragma unroll
            for (int i = 0; i < ORD; i++)
                a[i] = c == 0 ? w.wl[0][i] : (c == 1 ? w.wl[1][i] : w.wl[2][i]);
#pragma unroll
            for (int m = 0; m < NP; m++) {
                A0[m] = c == 0 ? w.s0[1][m] : w.s0[0][m];
                A1[m] = c == 0 ? w.s1[1][m] : w.s1[0][m];
            }
            const float B0 = c == 2 ? pick(w.s0[1], k) : pick(w.s0[2], k);
            const float B1 = c == 2 ? pick(w.s1[1], k) : pick(w.s1[2], k);
            const int si = c == 0 ? 3 : (c == 1 ? jsy : jsz);
            const int sm = c == 0 ? jsy : 3;
            const int sk = c == 2 ? jsy : jsz;
            const int o0 = c + sk * k;
#pragma unroll
            for (int m = 0; m < NP; m++) {
                const float wp = wperp(A0[m], A1[m], B0, B1);
#pragma unroll
                for (int i = 0; i < ORD; i++) {
                    const int o = o0 + si * i + sm * m;
                    fx_add(jl + o, jh + o, __float2int_rn(a[i] * wp), fx.shift);
                }
            }
        }
    }
}

// deposit the top entries of the warp's queue of 3D face crossings (up to 32 at a time, one
// per lane) while more than keep wait
template <int ORD>
__device__ __forceinline__ void segq_drain3(unsigned *Jl, unsigned *Jh, SegRec *sq,
                                            int &qn, int keep, const float *jn, int jsy,
                                            int jsz, FxFormat fx)
{
    const int lane = (int)(threadIdx.x & 31);
    while (qn > keep) {
        const int take = qn < 32 ? qn : 32, first = qn - take;
        __syncwarp();
        SegRec r{};
        const bool has = lane < take;
        if (has) r = sq[first + lane];
        qn = first;
        lanes_deposit3<ORD>(Jl, Jh, r, has, jn, jsy, jsz, fx);
    }
}

// ------------------------------------------------------------------------------------------
// 2D in-cell segments deposited into a global current array (the plain engine and the drop-in
// push): one segment per lane, base = offset of its stencil origin in J (-1: none).  Runs of
// lanes with one base (particles in cell order share cells) are summed per value through a
// per-warp scratch of 16 rows (column-major, stride SCR_LD), and lane k adds each run's sum of
// value k with one global atomic, instead of one atomic per particle and value.  Must be called
// by all 32 lanes; off[c] = offset of value lane + 32 c from the stencil origin.
// ------------------------------------------------------------------------------------------
template <typename T, int ORD>
__device__ __forceinline__ void cell_runs_deposit_global2(T *J, T *scr, long *sbase, long base,
                                                          const T *v, const int *off)
{
    constexpr int NV = SegVals<2, ORD>::NV;
    constexpr int NC = (NV + 31) / 32;
    const int lane = (int)(threadIdx.x & 31);
    const long prev = __shfl_up_sync(FULL_MASK, base, 1);
    const unsigned ends = __ballot_sync(FULL_MASK, lane > 0 && prev != base) >> 1;
    const long last = __shfl_sync(FULL_MASK, base, 31);
    T acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = T(0);
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if ((lane >> 4) == h) {
            const int r = lane & 15;
#pragma unroll
            for (int k = 0; k < NV; k++) scr[k * SCR_LD + r] = v[k];
            sbase[r] = base;
        }
        __syncwarp();
        const unsigned eh = (ends >> (16 * h)) & 0xffffu;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int col = lane + 32 * c;
            if (col < NV) {
                const T *cv = scr + col * SCR_LD;
                T a = acc[c];
#pragma unroll 1
                for (int r = 0; r < 16; r++) {
                    a += cv[r];
                    if (eh & (1u << r)) {
                        const long key = sbase[r];
                        if (key >= 0) atomicAdd(J + key + off[c], a);
                        a = T(0);
                    }
                }
                acc[c] = a;
            }
        }
        __syncwarp();
    }
    if (last >= 0) {
#pragma unroll
        for (int c = 0; c < NC; c++)
            if (lane + 32 * c < NV) atomicAdd(J + last + off[c], acc[c]);
    }
}

} // namespace osg
