// fft_radix.cuh -- in-register DFT butterflies of radix 2, 3, 4, 5, 8, 12, 16 used by
// the shared-memory Stockham FFTs (line filter and fused step).
//
// Radix<C2, R>::run<S>(a) replaces a[0..R) by y_q = sum_r a_r exp(S 2 pi i r q / R)
// with the direction S = -1 (forward) or +1 (inverse) fixed at compile time, so
// the multiplications by +-i fold into the additions; run(a, S) dispatches a
// runtime direction.
#pragma once

#include "clv_internal.cuh"

namespace clv {

// S * i * z for a compile-time direction S
template <int S, class C2>
__device__ __forceinline__ C2 times_si(C2 z) {
    C2 r;
    if (S > 0) { r.x = -z.y; r.y = z.x; }
    else { r.x = z.y; r.y = -z.x; }
    return r;
}

// Complex add/sub of the butterflies.  FP32 uses the packed two-lane FP32
// instructions of sm_100+ (add/sub .rn.f32x2: two IEEE single additions, the
// same results as the scalar pair), so one instruction moves a complex sum.
template <class C2> __device__ __forceinline__ C2 vadd(C2 a, C2 b) { return cadd(a, b); }
template <class C2> __device__ __forceinline__ C2 vsub(C2 a, C2 b) { return csub(a, b); }
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
template <> __device__ __forceinline__ float2 vadd<float2>(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
    return f2_unpack(r);
}
template <> __device__ __forceinline__ float2 vsub<float2>(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
    return f2_unpack(r);
}

template <class C2, int R>
struct Radix;

template <class C2>
struct Radix<C2, 2> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        C2 t = a[0];
        a[0] = vadd(t, a[1]);
        a[1] = vsub(t, a[1]);
    }
    static __device__ __forceinline__ void run(C2 *a, int) { run<1>(a); }
};

template <class C2>
struct Radix<C2, 4> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        const C2 s02 = vadd(a[0], a[2]), d02 = vsub(a[0], a[2]);
        const C2 s13 = vadd(a[1], a[3]), d13 = times_si<S>(vsub(a[1], a[3]));
        a[0] = vadd(s02, s13);
        a[2] = vsub(s02, s13);
        a[1] = vadd(d02, d13);
        a[3] = vsub(d02, d13);
    }
    static __device__ __forceinline__ void run(C2 *a, int S) {
        if (S < 0) run<-1>(a); else run<1>(a);
    }
};

template <class C2>
struct Radix<C2, 8> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        using R = decltype(a[0].x);
        const R h = (R)0.70710678118654752440;
        C2 e[4] = {a[0], a[2], a[4], a[6]};
        C2 o[4] = {a[1], a[3], a[5], a[7]};
        Radix<C2, 4>::template run<S>(e);
        Radix<C2, 4>::template run<S>(o);
        // twiddles exp(S 2 pi i q/8), q = 1, 2, 3
        C2 w1, w3;
        if (S < 0) {
            w1.x = h * (o[1].x + o[1].y); w1.y = h * (o[1].y - o[1].x);
            w3.x = h * (o[3].y - o[3].x); w3.y = -h * (o[3].x + o[3].y);
        } else {
            w1.x = h * (o[1].x - o[1].y); w1.y = h * (o[1].y + o[1].x);
            w3.x = -h * (o[3].x + o[3].y); w3.y = h * (o[3].x - o[3].y);
        }
        const C2 w2 = times_si<S>(o[2]);
        a[0] = vadd(e[0], o[0]); a[4] = vsub(e[0], o[0]);
        a[1] = vadd(e[1], w1);   a[5] = vsub(e[1], w1);
        a[2] = vadd(e[2], w2);   a[6] = vsub(e[2], w2);
        a[3] = vadd(e[3], w3);   a[7] = vsub(e[3], w3);
    }
    static __device__ __forceinline__ void run(C2 *a, int S) {
        if (S < 0) run<-1>(a); else run<1>(a);
    }
};

// z * w for a constant w = (wr, wi)
template <class C2, class R>
__device__ __forceinline__ C2 cmulc(C2 z, R wr, R wi) {
    C2 r;
    r.x = z.x * wr - z.y * wi;
    r.y = z.x * wi + z.y * wr;
    return r;
}

// 16 = 4 x 4: x[4 n1 + n2] -> radix 4 over n1 (index k1), twiddle W16^(n2 k1),
// radix 4 over n2 (index k2) -> X[k1 + 4 k2], W16 = exp(S 2 pi i / 16).
template <class C2>
struct Radix<C2, 16> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        using R = decltype(a[0].x);
        const R c = (R)0.92387953251128675613, s = (R)0.38268343236508977173;
        const R h = (R)0.70710678118654752440;
        const R sg = (R)S;
        C2 y[4][4];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            C2 t[4] = {a[n2], a[4 + n2], a[8 + n2], a[12 + n2]};
            Radix<C2, 4>::template run<S>(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = t[k1];
        }
        // W16^m = (cos(2 pi m/16), S sin(2 pi m/16))
        y[1][1] = cmulc(y[1][1], c, sg * s);   // m = 1
        y[1][2] = cmulc(y[1][2], h, sg * h);   // m = 2
        y[1][3] = cmulc(y[1][3], s, sg * c);   // m = 3
        y[2][1] = cmulc(y[2][1], h, sg * h);   // m = 2
        y[2][2] = times_si<S>(y[2][2]);        // m = 4
        y[2][3] = cmulc(y[2][3], -h, sg * h);  // m = 6
        y[3][1] = cmulc(y[3][1], s, sg * c);   // m = 3
        y[3][2] = cmulc(y[3][2], -h, sg * h);  // m = 6
        y[3][3] = cmulc(y[3][3], -c, -sg * s); // m = 9
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            C2 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
            Radix<C2, 4>::template run<S>(t);
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) a[k1 + 4 * k2] = t[k2];
        }
    }
    static __device__ __forceinline__ void run(C2 *a, int S) {
        if (S < 0) run<-1>(a); else run<1>(a);
    }
};

template <class C2>
struct Radix<C2, 3> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        using R = decltype(a[0].x);
        const R half = (R)0.5, s3 = (R)0.86602540378443864676;
        const C2 t1 = vadd(a[1], a[2]), t2 = vsub(a[1], a[2]);
        C2 m; m.x = a[0].x - half * t1.x; m.y = a[0].y - half * t1.y;
        const C2 r = times_si<S>(cscale(s3, t2));
        a[0] = vadd(a[0], t1);
        a[1] = vadd(m, r);
        a[2] = vsub(m, r);
    }
    static __device__ __forceinline__ void run(C2 *a, int S) {
        if (S < 0) run<-1>(a); else run<1>(a);
    }
};

// 12 = 4 x 3, coprime factors (Good-Thomas, no twiddles): x[(3 n1 + 4 n2) mod 12] ->
// radix 4 over n1 (index k1) for each n2, radix 3 over n2 (index k2) ->
// X[(9 k1 + 4 k2) mod 12], since (3 n1 + 4 n2)(9 k1 + 4 k2) = 3 n1 k1 + 4 n2 k2 mod 12.
template <class C2>
struct Radix<C2, 12> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        C2 y[3][4];
#pragma unroll
        for (int n2 = 0; n2 < 3; ++n2) {
            C2 t[4] = {a[(4 * n2) % 12], a[(3 + 4 * n2) % 12], a[(6 + 4 * n2) % 12], a[(9 + 4 * n2) % 12]};
            Radix<C2, 4>::template run<S>(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = t[k1];
        }
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            C2 t[3] = {y[0][k1], y[1][k1], y[2][k1]};
            Radix<C2, 3>::template run<S>(t);
#pragma unroll
            for (int k2 = 0; k2 < 3; ++k2) a[(9 * k1 + 4 * k2) % 12] = t[k2];
        }
    }
    static __device__ __forceinline__ void run(C2 *a, int S) {
        if (S < 0) run<-1>(a); else run<1>(a);
    }
};

template <class C2>
struct Radix<C2, 5> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        using R = decltype(a[0].x);
        const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;
        const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;
        const C2 t1 = vadd(a[1], a[4]), t2 = vadd(a[2], a[3]);
        const C2 t3 = vsub(a[1], a[4]), t4 = vsub(a[2], a[3]);
        C2 b1; b1.x = a[0].x + c1 * t1.x + c2 * t2.x; b1.y = a[0].y + c1 * t1.y + c2 * t2.y;
        C2 b2; b2.x = a[0].x + c2 * t1.x + c1 * t2.x; b2.y = a[0].y + c2 * t1.y + c1 * t2.y;
        C2 q1; q1.x = s1 * t3.x + s2 * t4.x; q1.y = s1 * t3.y + s2 * t4.y;
        C2 q2; q2.x = s2 * t3.x - s1 * t4.x; q2.y = s2 * t3.y - s1 * t4.y;
        q1 = times_si<S>(q1);
        q2 = times_si<S>(q2);
        a[0] = vadd(a[0], vadd(t1, t2));
        a[1] = vadd(b1, q1);
        a[4] = vsub(b1, q1);
        a[2] = vadd(b2, q2);
        a[3] = vsub(b2, q2);
    }
    static __device__ __forceinline__ void run(C2 *a, int S) {
        if (S < 0) run<-1>(a); else run<1>(a);
    }
};

// cos(2 pi m / 64) for m = 0 .. 16, and both parts of W64^m for any m by symmetry.
__host__ __device__ constexpr double cos64_quarter(int m) {
    switch (m) {
        case 0: return 1.0;
        case 1: return 0.995184726672196886245;
        case 2: return 0.980785280403230449126;
        case 3: return 0.956940335732208864936;
        case 4: return 0.923879532511286756128;
        case 5: return 0.881921264348355029713;
        case 6: return 0.831469612302545237079;
        case 7: return 0.773010453362736960811;
        case 8: return 0.707106781186547524401;
        case 9: return 0.634393284163645498215;
        case 10: return 0.555570233019602224743;
        case 11: return 0.471396736825997648556;
        case 12: return 0.382683432365089771728;
        case 13: return 0.290284677254462367636;
        case 14: return 0.195090322016128267848;
        case 15: return 0.0980171403295606019942;
        default: return 0.0;
    }
}
__host__ __device__ constexpr double cos64(int m) {
    m &= 63;
    return m <= 16 ? cos64_quarter(m) : (m <= 32 ? -cos64_quarter(32 - m) : (m <= 48 ? -cos64_quarter(m - 32) : cos64_quarter(64 - m)));
}
__host__ __device__ constexpr double sin64(int m) { return cos64((m + 48) & 63); }  // cos(2 pi (m - 16) / 64)

// 64 = 8 x 8: x[8 n1 + n2] -> radix 8 over n1 (index k1), twiddle W64^(n2 k1), radix 8
// over n2 (index k2) -> X[k1 + 8 k2], W64 = exp(S 2 pi i / 64); the twiddles are
// compile-time constants.  For a thread that holds a whole 64-site line in registers.
template <class C2>
struct Radix<C2, 64> {
    template <int S>
    static __device__ __forceinline__ void run(C2 *a) {
        using R = decltype(a[0].x);
        C2 y[8][8];
#pragma unroll
        for (int n2 = 0; n2 < 8; ++n2) {
            C2 t[8];
#pragma unroll
            for (int n1 = 0; n1 < 8; ++n1) t[n1] = a[8 * n1 + n2];
            Radix<C2, 8>::template run<S>(t);
#pragma unroll
            for (int k1 = 0; k1 < 8; ++k1) {
                const int m = n2 * k1;
                if (m == 0) y[n2][k1] = t[k1];
                else if (m == 16) y[n2][k1] = times_si<S>(t[k1]);
                else y[n2][k1] = cmulc(t[k1], (R)cos64(m), (R)(S * sin64(m)));
            }
        }
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) {
            C2 t[8];
#pragma unroll
            for (int n2 = 0; n2 < 8; ++n2) t[n2] = y[n2][k1];
            Radix<C2, 8>::template run<S>(t);
#pragma unroll
            for (int k2 = 0; k2 < 8; ++k2) a[k1 + 8 * k2] = t[k2];
        }
    }
};

}  // namespace clv
