// Shared-memory mixed-radix FFT convolution (see fftconv.cuh for the contract).
//
// 2-D data flow for one gradient evaluation (L = transform length, H = L/2 + 1):
//   k_kernel_rows  : builds the 4 kernel fields row by row (rows with a signed offset in
//                    (-M, M) only), r2c along the row, writes half spectra [4][L][H]
//   k_kernel_cols  : column FFTs of the kernel half spectra -> compact KSpec[H][L]
//   k_data_rows    : r2c of the M non-zero rows of the 4 spread fields -> [4][M][H]
//   k_data_cols    : per column: forward FFT (rows >= M are the zero padding), spectral
//                    products that form the 4 output fields, inverse FFT, keep rows < M
//   k_data_rows_inv: c2r of the M kept rows, keep columns < M -> potential grid
// Every pass keeps one or two whole transforms in shared memory; passes are Stockham
// (self-sorting) with radix 4, 2, 3, 5 butterflies.
#include <climits>
#include <map>
#include <mutex>

#include "fftconv.cuh"

namespace fitsne {

namespace {

template <typename C>
FITSNE_D C twid(const C *__restrict__ tw, int j, bool inv) {
    C w = tw[j];
    return inv ? cconj(w) : w;
}

// small DFTs; forward uses exp(-2 pi i / R), inverse exp(+2 pi i / R)
template <int R, typename C>
struct Dft;

template <typename C>
struct Dft<2, C> {
    static FITSNE_D void run(C *u, bool) {
        C a = u[0], b = u[1];
        u[0] = cadd(a, b);
        u[1] = csub(a, b);
    }
};

template <typename C>
struct Dft<4, C> {
    static FITSNE_D void run(C *u, bool inv) {
        C a0 = cadd(u[0], u[2]), a1 = csub(u[0], u[2]);
        C b0 = cadd(u[1], u[3]), b1 = csub(u[1], u[3]);
        C jb1 = inv ? cmul_pi(b1) : cmul_mi(b1);
        u[0] = cadd(a0, b0);
        u[2] = csub(a0, b0);
        u[1] = cadd(a1, jb1);
        u[3] = csub(a1, jb1);
    }
};

template <typename C>
struct Dft<3, C> {
    static FITSNE_D void run(C *u, bool inv) {
        typedef decltype(u[0].x) T;
        const T c = T(-0.5);
        const T s = T(0.86602540378443864676372317075294);  // sin(2 pi / 3)
        C t = cadd(u[1], u[2]);
        C d = csub(u[1], u[2]);
        C m = mkc(u[0].x + c * t.x, u[0].y + c * t.y);
        // forward: y1 = m - i s d, y2 = m + i s d
        C isd = mkc(-s * d.y, s * d.x);
        u[0] = cadd(u[0], t);
        if (!inv) {
            u[1] = csub(m, isd);
            u[2] = cadd(m, isd);
        } else {
            u[1] = cadd(m, isd);
            u[2] = csub(m, isd);
        }
    }
};

template <typename C>
struct Dft<5, C> {
    static FITSNE_D void run(C *u, bool inv) {
        typedef decltype(u[0].x) T;
        const T c1 = T(0.30901699437494742410229341718282);   // cos(2 pi / 5)
        const T s1 = T(0.95105651629515357211643933337938);   // sin(2 pi / 5)
        const T c2 = T(-0.80901699437494742410229341718282);  // cos(4 pi / 5)
        const T s2 = T(0.58778525229247312916870595463907);   // sin(4 pi / 5)
        C a1 = cadd(u[1], u[4]), b1 = csub(u[1], u[4]);
        C a2 = cadd(u[2], u[3]), b2 = csub(u[2], u[3]);
        C m1 = mkc(u[0].x + c1 * a1.x + c2 * a2.x, u[0].y + c1 * a1.y + c2 * a2.y);
        C m2 = mkc(u[0].x + c2 * a1.x + c1 * a2.x, u[0].y + c2 * a1.y + c1 * a2.y);
        // n1 = s1 b1 + s2 b2 ; n2 = s2 b1 - s1 b2 ; forward y1 = m1 - i n1, y4 = m1 + i n1,
        // y2 = m2 - i n2, y3 = m2 + i n2
        C n1 = mkc(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
        C n2 = mkc(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
        C in1 = cmul_pi(n1), in2 = cmul_pi(n2);
        u[0] = mkc(u[0].x + a1.x + a2.x, u[0].y + a1.y + a2.y);
        if (!inv) {
            u[1] = csub(m1, in1);
            u[4] = cadd(m1, in1);
            u[2] = csub(m2, in2);
            u[3] = cadd(m2, in2);
        } else {
            u[1] = cadd(m1, in1);
            u[4] = csub(m1, in1);
            u[2] = cadd(m2, in2);
            u[3] = csub(m2, in2);
        }
    }
};

// One Stockham butterfly: inputs i + r*T, twiddle exp(-+2 pi i r k / (p R)), outputs
// (i - k) R + k + r p with k = i mod p.
template <int R, typename C>
FITSNE_D void bfly(const C *src, C *dst, int i, int T, int p, int tws, const C *__restrict__ tw, bool inv) {
    const int k = i % p;
    C u[R];
#pragma unroll
    for (int r = 0; r < R; ++r) u[r] = src[i + r * T];
    if (k) {
#pragma unroll
        for (int r = 1; r < R; ++r) u[r] = cmul(u[r], twid(tw, r * k * tws, inv));
    }
    Dft<R, C>::run(u, inv);
    const int base = (i - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[base + r * p] = u[r];
}

// nf independent length-L transforms stored at a[f*L]; b is scratch of the same size.
// Data must be visible to the whole block on entry.  Returns the buffer holding the
// result (a or b).
template <typename C>
FITSNE_D C *fft_block(C *a, C *b, int nf, const FftPlan &pl, const C *__restrict__ tw, bool inv) {
    const int L = pl.L;
    C *src = a;
    C *dst = b;
    int p = 1;
    for (int s = 0; s < pl.nst; ++s) {
        const int R = pl.radix[s];
        const int T = L / R;
        const int tws = L / (p * R);
        const int total = T * nf;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int f = idx / T;
            const int i = idx - f * T;
            const C *sf = src + f * L;
            C *df = dst + f * L;
            if (R == 4)
                bfly<4>(sf, df, i, T, p, tws, tw, inv);
            else if (R == 2)
                bfly<2>(sf, df, i, T, p, tws, tw, inv);
            else if (R == 3)
                bfly<3>(sf, df, i, T, p, tws, tw, inv);
            else
                bfly<5>(sf, df, i, T, p, tws, tw, inv);
        }
        __syncthreads();
        C *t = src;
        src = dst;
        dst = t;
        p *= R;
    }
    return src;
}

// kernel values at node offset (dx, dy) in node units, node spacing h
template <typename T>
FITSNE_D void kernel_vals_2d(int dx, int dy, T h, T df, int mode, T &k, T &gx, T &gy, T &hh) {
    const T ex = T(dx) * h;
    const T ey = T(dy) * h;
    const T r2 = ex * ex + ey * ey;
    if (mode == KERNEL_DF1) {
        const T q = T(1) / (T(1) + r2);
        k = q * q;
        hh = k * r2;
    } else {
        const T base = T(1) + r2 / df;
        k = pow(base, -(df + T(1)));
        hh = pow(base, -df);
    }
    gx = k * ex;
    gy = k * ey;
}

template <typename T>
FITSNE_D void kernel_vals_1d(int d, T h, T df, int mode, T &k, T &g, T &hh) {
    const T e = T(d) * h;
    const T r2 = e * e;
    if (mode == KERNEL_DF1) {
        const T q = T(1) / (T(1) + r2);
        k = q * q;
        hh = k * r2;
    } else {
        const T base = T(1) + r2 / df;
        k = pow(base, -(df + T(1)));
        hh = pow(base, -df);
    }
    g = k * e;
}

// split the spectrum Z of (f + i g) into the half spectra of f and g at index kb
template <typename C, typename T>
FITSNE_D void unpack_r2c(const C *Zs, int L, int kb, C &F, C &G) {
    C Z = Zs[kb];
    C Zc = cconj(Zs[kb == 0 ? 0 : L - kb]);
    F = cscale(cadd(Z, Zc), T(0.5));
    G = cscale(cmul_mi(csub(Z, Zc)), T(0.5));
}

template <typename T>
FITSNE_D void kernel_rows_body(int r, int M, const FftPlan &pl, const typename Cx<T>::t *__restrict__ tw,
                               typename Cx<T>::t *__restrict__ krow, T h, T df, int mode) {
    typedef typename Cx<T>::t C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L, H = L / 2 + 1;
    C *bufa = reinterpret_cast<C *>(smem_raw);
    C *bufb = bufa + 2 * L;
    // rows dx = r >= 0 only: the fields are even in dx (K, Gy, H) or odd (Gx), so the
    // column pass reads row -dx as +-row dx
    const int a = r;
    const int dx = r;
    for (int b = threadIdx.x; b < L; b += blockDim.x) {
        T k = 0, gx = 0, gy = 0, hh = 0;
        if (b < M || b > L - M) {
            const int dy = (b < M) ? b : b - L;
            kernel_vals_2d<T>(dx, dy, h, df, mode, k, gx, gy, hh);
        }
        bufa[b] = mkc(k, gx);
        bufa[L + b] = mkc(gy, hh);
    }
    __syncthreads();
    C *res = fft_block(bufa, bufb, 2, pl, tw, false);
    for (int kb = threadIdx.x; kb < H; kb += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            C F, G;
            unpack_r2c<C, T>(res + q * L, L, kb, F, G);
            krow[((size_t) (2 * q) * L + a) * H + kb] = F;
            krow[((size_t) (2 * q + 1) * L + a) * H + kb] = G;
        }
    }
}

template <typename T>
__global__ void k_kernel_rows(int M, FftPlan pl, const typename Cx<T>::t *__restrict__ tw,
                              typename Cx<T>::t *__restrict__ krow, T h, T df, int mode,
                              const ConvGeom *__restrict__ cg) {
    if (cg) {
        M = cg->M;
        pl = cg->plan;
        h = (T) cg->h;
        if ((int) blockIdx.x >= M) return;
    }
    kernel_rows_body<T>(blockIdx.x, M, pl, tw, krow, h, df, mode);
}

template <typename T>
FITSNE_D void kernel_cols_body(int kb, int M, const FftPlan &pl, const typename Cx<T>::t *__restrict__ tw,
                               const typename Cx<T>::t *__restrict__ krow, KSpec<T> *__restrict__ kspec) {
    // The row spectra are real for K, Gx and H (even in dy) and imaginary for Gy (odd in dy);
    // as functions of dx, K, Gy and H are even and Gx is odd.  So one complex column FFT
    // carries K + i H (both outputs real: the real and imaginary parts) and another Gx + i Gy/i
    // (Gx's output imaginary and odd, Gy's real and even: split by the even / odd parts of
    // the imaginary output at k and L - k).
    typedef typename Cx<T>::t C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L, H = L / 2 + 1;
    C *z = reinterpret_cast<C *>(smem_raw);
    C *scratch = z + 2 * L;
    for (int a = threadIdx.x; a < L; a += blockDim.x) {
        C z1 = mkc(T(0), T(0)), z2 = mkc(T(0), T(0));
        const int idx = (a < M) ? a : ((a > L - M) ? L - a : -1);
        if (idx >= 0) {
            const T sgn = (a < M) ? T(1) : T(-1);  // Gx is odd in dx
            z1 = mkc(krow[((size_t) 0 * L + idx) * H + kb].x, krow[((size_t) 3 * L + idx) * H + kb].x);
            z2 = mkc(sgn * krow[((size_t) 1 * L + idx) * H + kb].x, krow[((size_t) 2 * L + idx) * H + kb].y);
        }
        z[a] = z1;
        z[L + a] = z2;
    }
    __syncthreads();
    const C *res = fft_block(z, scratch, 2, pl, tw, false);
    const T s = T(1) / (T(L) * T(L));
    for (int ka = threadIdx.x; ka < L; ka += blockDim.x) {
        const int km = ka ? L - ka : 0;
        const T i2 = res[L + ka].y, i2m = res[L + km].y;
        KSpec<T> e;
        e.k = res[ka].x * s;
        e.h = res[ka].y * s;
        e.gx = T(0.5) * (i2 - i2m) * s;
        e.gy = T(0.5) * (i2 + i2m) * s;
        kspec[(size_t) kb * L + ka] = e;
    }
}

template <typename T>
__global__ void k_kernel_cols(int M, FftPlan pl, const typename Cx<T>::t *__restrict__ tw,
                              const typename Cx<T>::t *__restrict__ krow, KSpec<T> *__restrict__ kspec,
                              const ConvGeom *__restrict__ cg) {
    if (cg) {
        M = cg->M;
        pl = cg->plan;
        if ((int) blockIdx.x >= pl.L / 2 + 1) return;
    }
    kernel_cols_body<T>(blockIdx.x, M, pl, tw, krow, kspec);
}

template <typename T>
FITSNE_D void data_rows_body(int a, const Cell4<T> *__restrict__ grid, int M, const FftPlan &pl,
                             const typename Cx<T>::t *__restrict__ tw, typename Cx<T>::t *__restrict__ d1) {
    typedef typename Cx<T>::t C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L, H = L / 2 + 1;
    C *bufa = reinterpret_cast<C *>(smem_raw);
    C *bufb = bufa + 2 * L;
    for (int b = threadIdx.x; b < L; b += blockDim.x) {
        Cell4<T> v;
        if (b < M)
            v = grid[(size_t) a * M + b];
        else
            v.a = v.b = v.c = v.d = T(0);
        bufa[b] = mkc(v.a, v.b);
        bufa[L + b] = mkc(v.c, v.d);
    }
    __syncthreads();
    C *res = fft_block(bufa, bufb, 2, pl, tw, false);
    for (int kb = threadIdx.x; kb < H; kb += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            C F, G;
            unpack_r2c<C, T>(res + q * L, L, kb, F, G);
            d1[((size_t) (2 * q) * M + a) * H + kb] = F;
            d1[((size_t) (2 * q + 1) * M + a) * H + kb] = G;
        }
    }
}

template <typename T>
__global__ void k_data_rows(const Cell4<T> *__restrict__ grid, int M, FftPlan pl,
                            const typename Cx<T>::t *__restrict__ tw, typename Cx<T>::t *__restrict__ d1,
                            const ConvGeom *__restrict__ cg) {
    if (cg) {
        M = cg->M;
        pl = cg->plan;
        if ((int) blockIdx.x >= M) return;
    }
    data_rows_body<T>(blockIdx.x, grid, M, pl, tw, d1);
}

template <typename T>
FITSNE_D void data_cols_body(int kb, int M, const FftPlan &pl, const typename Cx<T>::t *__restrict__ tw,
                             const typename Cx<T>::t *__restrict__ d1, const KSpec<T> *__restrict__ kspec,
                             typename Cx<T>::t *__restrict__ d2, int mode) {
    typedef typename Cx<T>::t C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L, H = L / 2 + 1;
    C *spec = reinterpret_cast<C *>(smem_raw);
    C *scratch = spec + 4 * L;
    // With room for eight transforms (the launch gives 8 L when it fits) the four fields go
    // through each Stockham stage together: a quarter of the stages' barriers and four times
    // the butterflies per stage for the block's threads.  Otherwise one field at a time with
    // one transform of scratch.  The butterflies are the same either way.
    unsigned dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const bool wide = (size_t) dyn >= 8 * (size_t) L * sizeof(C);
    for (int f = 0; f < 4; ++f)
        for (int a = threadIdx.x; a < L; a += blockDim.x)
            spec[f * L + a] = (a < M) ? d1[((size_t) f * M + a) * H + kb] : mkc(T(0), T(0));
    __syncthreads();
    C *fw = spec;  // the four forward spectra
    if (wide) {
        fw = fft_block(spec, scratch, 4, pl, tw, false);
    } else {
        for (int f = 0; f < 4; ++f) {
            C *res = fft_block(spec + f * L, scratch, 1, pl, tw, false);
            if (res != spec + f * L) {
                for (int a = threadIdx.x; a < L; a += blockDim.x) spec[f * L + a] = res[a];
                __syncthreads();
            }
        }
    }
    // spectral products forming V1, Rx, Ry and S (df = 1) or Vgen (variable df)
    for (int ka = threadIdx.x; ka < L; ka += blockDim.x) {
        const KSpec<T> e = kspec[(size_t) kb * L + ka];
        const C w1 = fw[ka], w2 = fw[L + ka], w3 = fw[2 * L + ka], w4 = fw[3 * L + ka];
        // (i g) w = (-g w.y, g w.x)
        const C gxw1 = mkc(-e.gx * w1.y, e.gx * w1.x);
        const C gyw1 = mkc(-e.gy * w1.y, e.gy * w1.x);
        const C v1 = cscale(w1, e.k);
        const C rx = csub(gxw1, cscale(w2, e.k));
        const C ry = csub(gyw1, cscale(w3, e.k));
        C s4;
        if (mode == KERNEL_DF1) {
            const C gxw2 = mkc(-e.gx * w2.y, e.gx * w2.x);
            const C gyw3 = mkc(-e.gy * w3.y, e.gy * w3.x);
            s4 = cadd(csub(cscale(w1, e.h), cscale(cadd(gxw2, gyw3), T(2))), cscale(w4, e.k));
        } else {
            s4 = cscale(w1, e.h);
        }
        fw[ka] = v1;
        fw[L + ka] = rx;
        fw[2 * L + ka] = ry;
        fw[3 * L + ka] = s4;
    }
    __syncthreads();
    if (wide) {
        const C *res = fft_block(fw, fw == spec ? scratch : spec, 4, pl, tw, true);
        for (int f = 0; f < 4; ++f)
            for (int a = threadIdx.x; a < M; a += blockDim.x) d2[((size_t) f * M + a) * H + kb] = res[f * L + a];
        return;
    }
    for (int f = 0; f < 4; ++f) {
        C *res = fft_block(spec + f * L, scratch, 1, pl, tw, true);
        for (int a = threadIdx.x; a < M; a += blockDim.x) d2[((size_t) f * M + a) * H + kb] = res[a];
        __syncthreads();
    }
}

// shared memory of the column pass: eight transforms when they fit (the four fields together)
template <typename C>
size_t data_cols_smem(int L) {
    const size_t s8 = 8 * (size_t) L * sizeof(C);
    return s8 <= 227 * 1024 ? s8 : 5 * (size_t) L * sizeof(C);
}

template <typename T>
__global__ void k_data_cols(int M, FftPlan pl, const typename Cx<T>::t *__restrict__ tw,
                            const typename Cx<T>::t *__restrict__ d1, const KSpec<T> *__restrict__ kspec,
                            typename Cx<T>::t *__restrict__ d2, int mode, const ConvGeom *__restrict__ cg) {
    if (cg) {
        M = cg->M;
        pl = cg->plan;
        if ((int) blockIdx.x >= pl.L / 2 + 1) return;
    }
    data_cols_body<T>(blockIdx.x, M, pl, tw, d1, kspec, d2, mode);
}

template <typename T>
FITSNE_D void data_rows_inv_body(int a, const typename Cx<T>::t *__restrict__ d2, int M, const FftPlan &pl,
                                 const typename Cx<T>::t *__restrict__ tw, Cell4<T> *__restrict__ out) {
    typedef typename Cx<T>::t C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L, H = L / 2 + 1;
    C *bufa = reinterpret_cast<C *>(smem_raw);
    C *bufb = bufa + 2 * L;
    for (int kb = threadIdx.x; kb < L; kb += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const C *rf = d2 + ((size_t) (2 * q) * M + a) * H;
            const C *rg = d2 + ((size_t) (2 * q + 1) * M + a) * H;
            C F, G;
            if (kb < H) {
                F = rf[kb];
                G = rg[kb];
            } else {
                F = cconj(rf[L - kb]);
                G = cconj(rg[L - kb]);
            }
            if (kb == 0 || 2 * kb == L) {
                F.y = T(0);
                G.y = T(0);
            }
            bufa[q * L + kb] = mkc(F.x - G.y, F.y + G.x);
        }
    }
    __syncthreads();
    C *res = fft_block(bufa, bufb, 2, pl, tw, true);
    for (int b = threadIdx.x; b < M; b += blockDim.x) {
        Cell4<T> v;
        v.a = res[b].x;
        v.b = res[b].y;
        v.c = res[L + b].x;
        v.d = res[L + b].y;
        out[(size_t) a * M + b] = v;
    }
}

template <typename T>
__global__ void k_data_rows_inv(const typename Cx<T>::t *__restrict__ d2, int M, FftPlan pl,
                                const typename Cx<T>::t *__restrict__ tw, Cell4<T> *__restrict__ out,
                                const ConvGeom *__restrict__ cg) {
    if (cg) {
        M = cg->M;
        pl = cg->plan;
        if ((int) blockIdx.x >= M) return;
    }
    data_rows_inv_body<T>(blockIdx.x, d2, M, pl, tw, out);
}

// ---- 1-D ----
template <typename T>
__global__ void k_conv1d_fwd(const Cell4<T> *__restrict__ grid, int M, FftPlan pl,
                             const typename Cx<T>::t *__restrict__ tw, typename Cx<T>::t *__restrict__ work, T h,
                             T df, int mode, const ConvGeom *__restrict__ cg) {
    typedef typename Cx<T>::t C;
    if (cg) {
        M = cg->M;
        pl = cg->plan;
        h = (T) cg->h;
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L;
    C *bufa = reinterpret_cast<C *>(smem_raw);
    C *bufb = bufa + L;
    const int f = blockIdx.x;  // 0..2 kernels (K, G, H|Kgen), 3..5 fields W1, W2', W3'
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        T v = 0;
        if (f < 3) {
            if (i < M || i > L - M) {
                T k, g, hh;
                kernel_vals_1d<T>(i < M ? i : i - L, h, df, mode, k, g, hh);
                v = (f == 0) ? k : ((f == 1) ? g : hh);
            }
        } else if (i < M) {
            const Cell4<T> c = grid[i];
            v = (f == 3) ? c.a : ((f == 4) ? c.b : c.c);
        }
        bufa[i] = mkc(v, T(0));
    }
    __syncthreads();
    C *res = fft_block(bufa, bufb, 1, pl, tw, false);
    for (int i = threadIdx.x; i < L; i += blockDim.x) work[(size_t) f * L + i] = res[i];
}

template <typename T>
__global__ void k_conv1d_inv(const typename Cx<T>::t *__restrict__ work, int M, FftPlan pl,
                             const typename Cx<T>::t *__restrict__ tw, Cell4<T> *__restrict__ out, int mode,
                             const ConvGeom *__restrict__ cg) {
    typedef typename Cx<T>::t C;
    if (cg) {
        M = cg->M;
        pl = cg->plan;
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = pl.L;
    C *bufa = reinterpret_cast<C *>(smem_raw);
    C *bufb = bufa + L;
    const int o = blockIdx.x;
    const T s = T(1) / T(L);
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        const T K = work[i].x * s;
        const T G = work[L + i].y * s;
        const T Hh = work[2 * L + i].x * s;
        const C w1 = work[3 * L + i], w2 = work[4 * L + i], w3 = work[5 * L + i];
        C v;
        if (o == 0) {
            v = cscale(w1, K);
        } else if (o == 1) {
            v = csub(mkc(-G * w1.y, G * w1.x), cscale(w2, K));
        } else if (mode == KERNEL_DF1) {
            v = cadd(csub(cscale(w1, Hh), cscale(mkc(-G * w2.y, G * w2.x), T(2))), cscale(w3, K));
        } else {
            v = cscale(w1, Hh);
        }
        bufa[i] = v;
    }
    __syncthreads();
    C *res = fft_block(bufa, bufb, 1, pl, tw, true);
    for (int i = threadIdx.x; i < M; i += blockDim.x) {
        T *cell = reinterpret_cast<T *>(out + i);
        cell[o] = res[i].x;
    }
}

// Raises a kernel's dynamic shared-memory limit to at least `bytes`, never lowers it: a launch
// recorded earlier in a CUDA graph for a larger transform (the iteration graphs are sized for
// the grid capacity) must stay valid after a smaller direct launch (the host-path step, the
// block-size timing), including when a profiler replays the graph's kernels one by one.
template <typename K>
cudaError_t set_smem(K kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<const void *, size_t> limit;
    std::lock_guard<std::mutex> lk(mu);
    size_t &cur = limit[reinterpret_cast<const void *>(kernel)];
    if (bytes <= cur || bytes <= 48 * 1024) return cudaSuccess;  // 48 KB need no attribute
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

}  // namespace

template <typename T>
cudaError_t conv2d_launch(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M, const FftPlan &plan,
                          const typename Cx<T>::t *tw, typename Cx<T>::t *work_a, typename Cx<T>::t *work_b,
                          KSpec<T> *kspec, double h, double df, int mode, cudaStream_t st, int threads) {
    typedef typename Cx<T>::t C;
    const int L = plan.L, H = L / 2 + 1;
    if (L > max_fft_len<T>() || L < 2 * M) return cudaErrorInvalidValue;
    const size_t s4 = 4 * (size_t) L * sizeof(C);
    const size_t s5 = 5 * (size_t) L * sizeof(C);
    cudaError_t e;
    if ((e = set_smem(k_kernel_rows<T>, s4)) != cudaSuccess) return e;
    if ((e = set_smem(k_kernel_cols<T>, s5)) != cudaSuccess) return e;
    if ((e = set_smem(k_data_rows<T>, s4)) != cudaSuccess) return e;
    const size_t sc = data_cols_smem<C>(L);
    if ((e = set_smem(k_data_cols<T>, sc)) != cudaSuccess) return e;
    if ((e = set_smem(k_data_rows_inv<T>, s4)) != cudaSuccess) return e;
    const int thr = (threads >= 32 && threads <= 1024 && threads % 32 == 0) ? threads : 256;
    // kernel spectra: krow uses work_a ([4][L][H]); data passes use work_b ([4][M][H]) then work_a
    k_kernel_rows<T><<<M, thr, s4, st>>>(M, plan, tw, work_a, (T) h, (T) df, mode, nullptr);
    k_kernel_cols<T><<<H, thr, s5, st>>>(M, plan, tw, work_a, kspec, nullptr);
    k_data_rows<T><<<M, thr, s4, st>>>(grid_in, M, plan, tw, work_b, nullptr);
    k_data_cols<T><<<H, thr, sc, st>>>(M, plan, tw, work_b, kspec, work_a, mode, nullptr);
    k_data_rows_inv<T><<<M, thr, s4, st>>>(work_a, M, plan, tw, grid_out, nullptr);
    return cudaGetLastError();
}

template <typename T>
cudaError_t conv2d_launch_dev(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M_cap, int L_cap, const ConvGeom *cg,
                              const typename Cx<T>::t *tw, typename Cx<T>::t *work_a, typename Cx<T>::t *work_b,
                              KSpec<T> *kspec, double df, int mode, cudaStream_t st, int threads) {
    typedef typename Cx<T>::t C;
    const int H = L_cap / 2 + 1;
    if (L_cap > max_fft_len<T>() || L_cap < 2 * M_cap) return cudaErrorInvalidValue;
    const size_t s4 = 4 * (size_t) L_cap * sizeof(C);
    const size_t s5 = 5 * (size_t) L_cap * sizeof(C);
    cudaError_t e;
    if ((e = set_smem(k_kernel_rows<T>, s4)) != cudaSuccess) return e;
    if ((e = set_smem(k_kernel_cols<T>, s5)) != cudaSuccess) return e;
    if ((e = set_smem(k_data_rows<T>, s4)) != cudaSuccess) return e;
    const size_t sc = data_cols_smem<C>(L_cap);
    if ((e = set_smem(k_data_cols<T>, sc)) != cudaSuccess) return e;
    if ((e = set_smem(k_data_rows_inv<T>, s4)) != cudaSuccess) return e;
    const int thr = (threads >= 32 && threads <= 1024 && threads % 32 == 0) ? threads : 256;
    FftPlan dummy{};
    k_kernel_rows<T><<<M_cap, thr, s4, st>>>(0, dummy, tw, work_a, T(0), (T) df, mode, cg);
    k_kernel_cols<T><<<H, thr, s5, st>>>(0, dummy, tw, work_a, kspec, cg);
    k_data_rows<T><<<M_cap, thr, s4, st>>>(grid_in, 0, dummy, tw, work_b, cg);
    k_data_cols<T><<<H, thr, sc, st>>>(0, dummy, tw, work_b, kspec, work_a, mode, cg);
    k_data_rows_inv<T><<<M_cap, thr, s4, st>>>(work_a, 0, dummy, tw, grid_out, cg);
    return cudaGetLastError();
}

template <typename T>
cudaError_t conv1d_launch(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M, const FftPlan &plan,
                          const typename Cx<T>::t *tw, typename Cx<T>::t *work, double h, double df, int mode,
                          cudaStream_t st) {
    typedef typename Cx<T>::t C;
    const int L = plan.L;
    const size_t s2 = 2 * (size_t) L * sizeof(C);
    if (L < 2 * M || s2 > 227 * 1024) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = set_smem(k_conv1d_fwd<T>, s2)) != cudaSuccess) return e;
    if ((e = set_smem(k_conv1d_inv<T>, s2)) != cudaSuccess) return e;
    k_conv1d_fwd<T><<<6, 512, s2, st>>>(grid_in, M, plan, tw, work, (T) h, (T) df, mode, nullptr);
    k_conv1d_inv<T><<<3, 512, s2, st>>>(work, M, plan, tw, grid_out, mode, nullptr);
    return cudaGetLastError();
}

template <typename T>
cudaError_t conv1d_launch_dev(const Cell4<T> *grid_in, Cell4<T> *grid_out, int L_cap, const ConvGeom *cg,
                              const typename Cx<T>::t *tw, typename Cx<T>::t *work, double df, int mode,
                              cudaStream_t st) {
    typedef typename Cx<T>::t C;
    const size_t s2 = 2 * (size_t) L_cap * sizeof(C);
    if (s2 > 227 * 1024) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = set_smem(k_conv1d_fwd<T>, s2)) != cudaSuccess) return e;
    if ((e = set_smem(k_conv1d_inv<T>, s2)) != cudaSuccess) return e;
    FftPlan dummy{};
    k_conv1d_fwd<T><<<6, 512, s2, st>>>(grid_in, 0, dummy, tw, work, T(0), (T) df, mode, cg);
    k_conv1d_inv<T><<<3, 512, s2, st>>>(work, 0, dummy, tw, grid_out, mode, cg);
    return cudaGetLastError();
}

namespace {
template <typename T>
__global__ void k_twiddles_geom(const ConvGeom *__restrict__ cg, typename Cx<T>::t *__restrict__ tw) {
    const int L = cg->plan.L;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        double sn, cs;
        sincospi(2.0 * (double) j / (double) L, &sn, &cs);
        tw[j] = mkc((T) cs, (T) -sn);
    }
}
}  // namespace

template <typename T>
cudaError_t twiddles_dev(const ConvGeom *cg, typename Cx<T>::t *tw, cudaStream_t st) {
    k_twiddles_geom<T><<<8, 256, 0, st>>>(cg, tw);
    return cudaGetLastError();
}

// ---- batched 2-D convolution: one launch per pass for all jobs ----
namespace {
template <typename T>
__global__ void k_bkernel_rows(FftBatchMap m, const FftBatchJob *__restrict__ jobs,
                               const typename Cx<T>::t *__restrict__ tw, typename Cx<T>::t *__restrict__ work_a, T df,
                               int mode) {
    const int j = m.job[blockIdx.x];
    const FftBatchJob jb = jobs[j];
    const int M = jb.cg->M;
    const FftPlan pl = jb.cg->plan;
    const int r = (int) blockIdx.x - m.first[j];
    if (r >= M) return;
    kernel_rows_body<T>(r, M, pl, tw + jb.tw0, work_a + jb.work0, (T) jb.cg->h, df, mode);
}

template <typename T>
__global__ void k_bkernel_cols(FftBatchMap m, const FftBatchJob *__restrict__ jobs,
                               const typename Cx<T>::t *__restrict__ tw, const typename Cx<T>::t *__restrict__ work_a,
                               KSpec<T> *__restrict__ kspec) {
    const int j = m.job[blockIdx.x];
    const FftBatchJob jb = jobs[j];
    const int M = jb.cg->M;
    const FftPlan pl = jb.cg->plan;
    const int kb = (int) blockIdx.x - m.first[j];
    if (kb >= pl.L / 2 + 1) return;
    kernel_cols_body<T>(kb, M, pl, tw + jb.tw0, work_a + jb.work0, kspec + jb.kspec0);
}

template <typename T>
__global__ void k_bdata_rows(FftBatchMap m, const FftBatchJob *__restrict__ jobs, const Cell4<T> *__restrict__ grid,
                             const typename Cx<T>::t *__restrict__ tw, typename Cx<T>::t *__restrict__ work_b) {
    const int j = m.job[blockIdx.x];
    const FftBatchJob jb = jobs[j];
    const int M = jb.cg->M;
    const FftPlan pl = jb.cg->plan;
    const int a = (int) blockIdx.x - m.first[j];
    if (a >= M) return;
    data_rows_body<T>(a, grid + jb.cell0, M, pl, tw + jb.tw0, work_b + jb.work0);
}

template <typename T>
__global__ void k_bdata_cols(FftBatchMap m, const FftBatchJob *__restrict__ jobs,
                             const typename Cx<T>::t *__restrict__ tw, const typename Cx<T>::t *__restrict__ work_b,
                             const KSpec<T> *__restrict__ kspec, typename Cx<T>::t *__restrict__ work_a, int mode) {
    const int j = m.job[blockIdx.x];
    const FftBatchJob jb = jobs[j];
    const int M = jb.cg->M;
    const FftPlan pl = jb.cg->plan;
    const int kb = (int) blockIdx.x - m.first[j];
    if (kb >= pl.L / 2 + 1) return;
    data_cols_body<T>(kb, M, pl, tw + jb.tw0, work_b + jb.work0, kspec + jb.kspec0, work_a + jb.work0, mode);
}

template <typename T>
__global__ void k_bdata_rows_inv(FftBatchMap m, const FftBatchJob *__restrict__ jobs,
                                 const typename Cx<T>::t *__restrict__ work_a, const typename Cx<T>::t *__restrict__ tw,
                                 Cell4<T> *__restrict__ out) {
    const int j = m.job[blockIdx.x];
    const FftBatchJob jb = jobs[j];
    const int M = jb.cg->M;
    const FftPlan pl = jb.cg->plan;
    const int a = (int) blockIdx.x - m.first[j];
    if (a >= M) return;
    data_rows_inv_body<T>(a, work_a + jb.work0, M, pl, tw + jb.tw0, out + jb.cell0);
}

// job blockIdx.y's twiddles for its current length
template <typename T>
__global__ void k_btwiddles(const FftBatchJob *__restrict__ jobs, typename Cx<T>::t *__restrict__ tw) {
    const FftBatchJob jb = jobs[blockIdx.y];
    const int L = jb.cg->plan.L;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        double sn, cs;
        sincospi(2.0 * (double) k / (double) L, &sn, &cs);
        tw[jb.tw0 + k] = mkc((T) cs, (T) -sn);
    }
}
}  // namespace

template <typename T>
cudaError_t conv2d_launch_batch(const Cell4<T> *grid_in, Cell4<T> *grid_out, const FftBatchJob *jobs,
                                FftBatchMap krow, int nkrow, FftBatchMap cols, int ncols, FftBatchMap rows, int nrows,
                                int L_max, const typename Cx<T>::t *tw, typename Cx<T>::t *work_a,
                                typename Cx<T>::t *work_b, KSpec<T> *kspec, double df, int mode, cudaStream_t st) {
    typedef typename Cx<T>::t C;
    if (L_max > max_fft_len<T>()) return cudaErrorInvalidValue;
    const size_t s4 = 4 * (size_t) L_max * sizeof(C);
    const size_t s5 = 5 * (size_t) L_max * sizeof(C);
    cudaError_t e;
    if ((e = set_smem(k_bkernel_rows<T>, s4)) != cudaSuccess) return e;
    if ((e = set_smem(k_bkernel_cols<T>, s5)) != cudaSuccess) return e;
    if ((e = set_smem(k_bdata_rows<T>, s4)) != cudaSuccess) return e;
    const size_t sc = data_cols_smem<C>(L_max);
    if ((e = set_smem(k_bdata_cols<T>, sc)) != cudaSuccess) return e;
    if ((e = set_smem(k_bdata_rows_inv<T>, s4)) != cudaSuccess) return e;
    const int thr = 256;
    k_bkernel_rows<T><<<nkrow, thr, s4, st>>>(krow, jobs, tw, work_a, (T) df, mode);
    k_bkernel_cols<T><<<ncols, thr, s5, st>>>(cols, jobs, tw, work_a, kspec);
    k_bdata_rows<T><<<nrows, thr, s4, st>>>(rows, jobs, grid_in, tw, work_b);
    k_bdata_cols<T><<<ncols, thr, sc, st>>>(cols, jobs, tw, work_b, kspec, work_a, mode);
    k_bdata_rows_inv<T><<<nrows, thr, s4, st>>>(rows, jobs, work_a, tw, grid_out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t twiddles_batch(const FftBatchJob *jobs, int J, typename Cx<T>::t *tw, cudaStream_t st) {
    k_btwiddles<T><<<dim3(4, J), 256, 0, st>>>(jobs, tw);
    return cudaGetLastError();
}

template cudaError_t conv2d_launch_batch<float>(const Cell4<float> *, Cell4<float> *, const FftBatchJob *,
                                                FftBatchMap, int, FftBatchMap, int, FftBatchMap, int, int,
                                                const float2 *, float2 *, float2 *, KSpec<float> *, double, int,
                                                cudaStream_t);
template cudaError_t twiddles_batch<float>(const FftBatchJob *, int, float2 *, cudaStream_t);

template cudaError_t conv2d_launch<float>(const Cell4<float> *, Cell4<float> *, int, const FftPlan &, const float2 *,
                                          float2 *, float2 *, KSpec<float> *, double, double, int, cudaStream_t, int);
template cudaError_t conv2d_launch<double>(const Cell4<double> *, Cell4<double> *, int, const FftPlan &,
                                           const double2 *, double2 *, double2 *, KSpec<double> *, double, double,
                                           int, cudaStream_t, int);
template cudaError_t conv1d_launch<float>(const Cell4<float> *, Cell4<float> *, int, const FftPlan &, const float2 *,
                                          float2 *, double, double, int, cudaStream_t);
template cudaError_t conv1d_launch<double>(const Cell4<double> *, Cell4<double> *, int, const FftPlan &,
                                           const double2 *, double2 *, double, double, int, cudaStream_t);
template cudaError_t conv2d_launch_dev<float>(const Cell4<float> *, Cell4<float> *, int, int, const ConvGeom *,
                                              const float2 *, float2 *, float2 *, KSpec<float> *, double, int,
                                              cudaStream_t, int);
template cudaError_t conv2d_launch_dev<double>(const Cell4<double> *, Cell4<double> *, int, int, const ConvGeom *,
                                               const double2 *, double2 *, double2 *, KSpec<double> *, double, int,
                                               cudaStream_t, int);
template cudaError_t conv1d_launch_dev<float>(const Cell4<float> *, Cell4<float> *, int, const ConvGeom *,
                                              const float2 *, float2 *, double, int, cudaStream_t);
template cudaError_t conv1d_launch_dev<double>(const Cell4<double> *, Cell4<double> *, int, const ConvGeom *,
                                               const double2 *, double2 *, double, int, cudaStream_t);
template cudaError_t twiddles_dev<float>(const ConvGeom *, float2 *, cudaStream_t);
template cudaError_t twiddles_dev<double>(const ConvGeom *, double2 *, cudaStream_t);

}  // namespace fitsne
