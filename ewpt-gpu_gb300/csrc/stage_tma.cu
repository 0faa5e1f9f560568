// stage_tma.cu -- FP32-form RK4 stage kernel on TMA-staged shared-memory tiles.
//
// Same stage structure, physics and arithmetic as k_stage_fp32x2
// (stage_pair.cu: two x-adjacent sites per thread in packed FP32x2), but the
// stencil operands come from shared memory.  A CTA owns a tile of
// 32 x by x 4 sites (by = 4 or 2): 16*by*4 compute threads and one producer
// warp.  The physics (physics.cuh) consumes the stage-input arrays in a fixed
// order -- the 12 momentum arrays of the Gauss-law divergences (one axis
// each), then the 20 field arrays (gradient, mostly with the Laplacian) --
// and the kernel streams exactly that sequence of 32 boxes through an 8-slot
// ring in shared memory:
//   * each box is one cp.async.bulk.tensor (TMA) copy of the tile plus its
//     3-site halo out of the ghosted layout (ewpt_internal.cuh), whose ghost
//     cells already hold the periodic images, so a box never wraps: full
//     boxes (32+8) x (by+6) x (4+6) for the field arrays, one-axis boxes
//     (halo along x, y or z only) for the momentum arrays;
//   * per slot a "full" mbarrier (the copy's transaction bytes) and an
//     "empty" mbarrier (one arrival per compute warp once it has read the box);
//   * lane 0 of the producer warp walks the boxes of every tile of the CTA
//     (the grid is persistent, one CTA per SM) and issues box g as soon as
//     the compute warps have released box g-8, so copies run up to 7 boxes
//     ahead of the arithmetic, across tile boundaries.
// After each stage k_ghost_fill refreshes the ghost images of what it wrote,
// so the next stage's boxes are ready.  A separate producer warp matters:
// with thread 0 of the compute warps refilling the ring, the kernel ran at
// half the speed.
//
// Every mbarrier wait is bounded, by the context's wait limit (polls;
// ewpt_set_wait_limit, default kSpin).  A compute thread whose wait runs out
// sets the context's error word and runs to the end without further waits
// or releases (results invalid, reported as EWPT_ERR_TIMEOUT by the host):
// a warp releases a slot only after it saw that slot's copy land, so the
// producer never issues a copy into a slot whose previous copy may still be
// in flight.  A producer whose wait for a free slot runs out stops issuing;
// it then waits for its last copies to land, always with the full kSpin
// limit, before it exits, so no copy outlives the CTA.
#include <cuda.h>

#include <mutex>

#include "accessors.cuh"
#include "ewpt_ctx.cuh"

namespace {

constexpr int BX = 32;                       // tile extent along x in sites (16 threads, two sites each)
constexpr int FX = BX + 8;                   // box extent along x with the halo
constexpr int NS = 8;                        // ring slots
constexpr int NSTEN = 32;                    // stencil boxes per tile
constexpr long kSpin = 1L << 22;             // try_wait polls before a wait gives up
// Stream the epilogue operands (kacc, y_hi, y_lo at the tile's sites) through
// the ring as well.  Measured on GB300 at 256^3: 18.2 ms per step against
// 14.3 ms with plain global loads -- the 16-24 extra boxes per tile make the
// 8-slot ring the bottleneck -- so the global loads are kept.  (Pulling the
// next tile's operands into L2 ahead of time, by TMA prefetch or by the idle
// producer lanes, was slower still: 16.4 and 16.8 ms.)
constexpr bool kEpilogueInRing = false;

// The box sequence of one tile for a stage whose epilogue reads NB buffers
// at the tile's own sites (stage 1: none; 2, 3: RK4 accumulator and state
// high part; 4: also the state low part).  The epilogue boxes hold the
// tile's sites of groups of arrays in the order the physics emits its rates
// (0-7, 8-15, 16, 17, 18, 19, 20-27, 28-35) and are placed in the sequence
// right where each group's rates come out, so every box is read, and
// released, shortly after it arrives (the ring is first in, first out):
//   E0 E1 | s0 s1 s2 | E2 | s3 s4 s5 | E3 | s6 s7 s8 | E4 | s9 s10 s11 | E5 |
//   s12 .. s31 | E6 E7        (each E* = NB boxes, one per buffer)
template <int NB>
struct Seq {
    static constexpr int NLOAD = NSTEN + 8 * NB;
    static_assert(NLOAD % NS == 0, "slot of box j must not depend on the tile");
    // position of stencil box s
    __host__ __device__ static constexpr int sten(int s) {
        return s + NB * (2 + (s >= 3) + (s >= 6) + (s >= 9) + (s >= 12));
    }
    // position of epilogue group g, buffer b
    __host__ __device__ static constexpr int epi(int g, int b) {
        return g == 0 ? b
               : g == 1 ? NB + b
               : g <= 5 ? 3 * (g - 1) + g * NB + b
                        : NSTEN + g * NB + b;
    }
    // what sits at position j: stencil box (returns s >= 0) or epilogue
    // group g, buffer b (returns -1)
    __host__ __device__ static int decode(int j, int& g, int& b) {
        for (int q = 0; q < NSTEN; ++q)
            if (sten(q) == j) return q;
        for (g = 0; g < 8; ++g)
            for (b = 0; b < NB; ++b)
                if (epi(g, b) == j) return -1;
        return -2;
    }
};
// epilogue groups: first array and size
__host__ __device__ constexpr int group_of(int a) { return a < 8 ? 0 : a < 16 ? 1 : a < 20 ? 2 + (a - 16) : a < 28 ? 6 : 7; }
__host__ __device__ constexpr int group_first(int g) { return g == 0 ? 0 : g == 1 ? 8 : g <= 5 ? 14 + g : g == 6 ? 20 : 28; }
__host__ __device__ constexpr int group_size(int g) { return g <= 1 || g >= 6 ? 8 : 1; }

// Tile of BX x TBY x TBZ sites: 16*TBY*TBZ compute threads plus one
// producer warp whose lane 0 issues every copy.
template <int TBY, int TBZ>
struct Cfg {
    static constexpr int BY = TBY, BZ = TBZ;
    static constexpr int NT = (BX / 2) * BY * BZ;
    static constexpr int NTHREADS = NT + 32;
    static constexpr int NWARP = NT / 32;
    static constexpr int FY = BY + 6, FZ = BZ + 6;
    static constexpr int TILE = BX * BY * BZ;  // sites of one array in a tile
    static constexpr int SLOT_FLOATS = FX * FY * FZ > 8 * TILE ? FX * FY * FZ : 8 * TILE;
    static constexpr int SMEM_BYTES = NS * SLOT_FLOATS * 4 + 128;
    static_assert((SLOT_FLOATS * 4) % 128 == 0, "slots must stay 128-byte aligned");
    static_assert(NT % 32 == 0, "whole warps");
};

enum Box { BOX_X = 0, BOX_Y = 1, BOX_Z = 2, BOX_FULL = 3 };

// box j of a tile: the array it holds and its shape
__host__ __device__ constexpr int load_array(int j) {
    return j < 12 ? 24 + j : (j < 25 ? j - 12 : (j < 28 ? j - 9 : (j < 31 ? j - 15 : 19)));
}
__host__ __device__ constexpr int load_box(int j) { return j < 12 ? j % 3 : BOX_FULL; }
template <class C>
__host__ __device__ constexpr uint32_t box_bytes(int box) {
    return box == BOX_FULL ? FX * C::FY * C::FZ * 4
                           : box == BOX_X ? FX * C::BY * C::BZ * 4 : box == BOX_Y ? BX * C::FY * C::BZ * 4
                                                                                  : BX * C::BY * C::FZ * 4;
}
// index of the box that holds field array a (0..19) in full
__device__ __forceinline__ constexpr int full_seq(int a) {
    return a <= 12 ? a + 12 : (a <= 15 ? a + 15 : (a <= 18 ? a + 9 : 31));
}

struct TmaMaps {
    CUtensorMap m[4];  // BOX_X, BOX_Y, BOX_Z, BOX_FULL over [36][pz][py][px] floats
};
// tile boxes of 8 and of 1 array(s) of the epilogue buffers: [buffer][0: 8, 1: 1]
struct EpiMaps {
    CUtensorMap m[3][2];
};

// ------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Compute-warp side.  The waits, the shared-memory reads and the releases
// carry no compiler memory clobber, so the compiler stays free to schedule
// the global loads of centres and epilogue operands early (as in the kernels
// that read every operand from global memory); their order is kept by data
// dependencies instead: a wait returns an opaque zero that is added to every
// shared address read from that box, and a release takes a value computed
// from those reads.  The hardware order comes from the acquire semantics of
// try_wait and the release semantics of arrive.
__device__ __forceinline__ uint32_t mbar_test_nc(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity));
    return ok;
}
__device__ __forceinline__ uint32_t opaque_zero(uint32_t dep) {
    uint32_t z;
    asm volatile("mov.u32 %0, 0;" : "=r"(z) : "r"(dep));
    return z;
}
__device__ __forceinline__ float2 lds2(uint32_t addr) {
    float2 v;
    asm("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}
__device__ __forceinline__ void warp_sync_after(float dep) {
    asm volatile("bar.warp.sync -1;" ::"f"(dep));
}
__device__ __forceinline__ void mbar_arrive_nc(uint32_t bar, float dep) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar), "f"(dep));
}
// bounded wait for the phase of the given parity
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long spin) {
    for (long it = 0; it < spin; ++it)
        if (mbar_test(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

// ------------------------------------------------------------- the ring
template <class C, int NB>
struct Ring {
    using S = Seq<NB>;
    uint32_t slots;   // shared-window address of slot 0
    uint32_t bars;    // full[NS] then empty[NS]
    const TmaMaps* maps;
    const EpiMaps* emaps;
    int* err;
    long spin;               // polls before a wait gives up (the drain uses kSpin)
    int ntx, nty, ntiles;
    int x0, y0, z0;          // box origin (padded coordinates) of the current tile
    uint32_t tpar;           // parity offset of the current tile's boxes
    mutable int ok;          // no wait has run out

    // tile t of the chunked walk (chunk_walk, y chunks of kChunkRows rows)
    __device__ __forceinline__ void origin(int t, int& x, int& y, int& z) const {
        int tx, ty, tz;
        chunk_walk(t, ntx, nty, ntiles / (ntx * nty), kChunkRows / C::BY, tx, ty, tz);
        x = tx * BX;
        y = ty * C::BY;
        z = tz * C::BZ;
    }
    __device__ __forceinline__ void set_tile(int t, int iter) {
        origin(t, x0, y0, z0);
        tpar = (uint32_t)(iter * (S::NLOAD / NS)) & 1u;
    }

    __device__ __forceinline__ uint32_t full(int s) const { return bars + 8 * s; }
    __device__ __forceinline__ uint32_t empty(int s) const { return bars + 8 * (NS + s); }

    // producer: issue the box at position j of the tile with box origin (ox, oy, oz)
    __device__ __forceinline__ void issue(int ox, int oy, int oz, int j) const {
        const int s = j % NS;
        int g = 0, b = 0;
        const int q = S::decode(j, g, b);
        if (q >= 0) {
            const int box = load_box(q);
            const int cx = box == BOX_FULL || box == BOX_X ? ox : ox + 4;
            const int cy = box == BOX_FULL || box == BOX_Y ? oy : oy + 3;
            const int cz = box == BOX_FULL || box == BOX_Z ? oz : oz + 3;
            mbar_expect_tx(full(s), box_bytes<C>(box));
            tma_load_4d(slots + s * C::SLOT_FLOATS * 4, &maps->m[box], cx, cy, cz, load_array(q), full(s));
        } else {
            const int n = group_size(g);
            mbar_expect_tx(full(s), n * C::TILE * 4);
            tma_load_4d(slots + s * C::SLOT_FLOATS * 4, &emaps->m[b][n == 8 ? 0 : 1], ox + 4, oy + 3, oz + 3,
                        group_first(g), full(s));
        }
    }
    // wait for box j; returns the shared address of its slot (with the
    // opaque dependency folded in)
    __device__ __forceinline__ uint32_t wait_box(int j) const {
        uint32_t got = 1;
        if (ok) {
            got = 0;
            const uint32_t par = ((uint32_t)(j / NS) & 1u) ^ tpar;
            for (long it = 0; it < spin && !got; ++it) got = mbar_test_nc(full(j % NS), par);
            if (!got) {
                ok = 0;
                atomicExch(err, 1);
            }
        }
        return slots + (j % NS) * C::SLOT_FLOATS * 4 + opaque_zero(got);
    }
    // this warp is done with box j (dep: a value computed from its reads);
    // after a wait of lane 0 ran out the warp releases nothing more
    __device__ __forceinline__ void release(int j, float dep) const {
        warp_sync_after(dep);
        if ((threadIdx.x & 31) == 0 && ok) mbar_arrive_nc(empty(j % NS), dep);
    }
    // producer warp, lane 0: every box of every tile of this CTA, each as soon
    // as the compute warps have released the previous occupant of its slot;
    // then wait for the last copies to land
    __device__ void produce() {
        int gq = 0;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            int ox, oy, oz;
            origin(t, ox, oy, oz);
            for (int j = 0; j < S::NLOAD; ++j, ++gq) {
                if (gq >= NS && !mbar_wait(empty(j % NS), ((gq / NS) + 1) & 1, spin)) {
                    ok = 0;
                    atomicExch(err, 3);
                    break;
                }
                issue(ox, oy, oz, j);
            }
        }
        for (int q = gq - 1; q >= 0 && q >= gq - NS; --q) mbar_wait(full(q % NS), (q / NS) & 1, kSpin);
    }
};

// ------------------------------------------------------------- accessor
// Two x-adjacent sites (lx, lx+1) of the tile; same stencil arithmetic as
// PairAcc, operands from the ring's slots (shared-window byte addresses).
template <class C, int NB>
struct TmaAcc {
    using S = Seq<NB>;
    static constexpr int BY = C::BY, BZ = C::BZ, FY = C::FY, FZ = C::FZ;
    const Ring<C, NB>& R;
    const float* X;  // stage input (centre values), ghosted layout
    int64_t P;
    int c;           // ghosted index of site lx
    int lx, ly, lz;
    StencilCoef<f2> s;

    __device__ __forceinline__ f2 v(int a) const {
        return f2(__ldg(reinterpret_cast<const float2*>(X + a * P + c)));
    }
    __device__ __forceinline__ static f2 l2(uint32_t a) { return f2(lds2(a)); }
    // x pairs around the centre q of a row with x halo 4
    __device__ __forceinline__ static void xpairs(uint32_t q, f2& p1, f2& p2, f2& p3, f2& m1, f2& m2, f2& m3) {
        const float2 qm2 = lds2(q - 16), qm1 = lds2(q - 8), q0 = lds2(q), qp1 = lds2(q + 8), qp2 = lds2(q + 16);
        p1 = f2(make_float2(q0.y, qp1.x));
        p2 = f2(qp1);
        p3 = f2(make_float2(qp1.y, qp2.x));
        m1 = f2(make_float2(qm1.y, q0.x));
        m2 = f2(qm1);
        m3 = f2(make_float2(qm2.y, qm1.x));
    }
    // 6th-order first derivative along a stride of st floats
    __device__ __forceinline__ f2 d1(uint32_t q, int st) const {
        const int b = 4 * st;
        return s.a1 * (l2(q + b) - l2(q - b)) + s.a2 * (l2(q + 2 * b) - l2(q - 2 * b)) +
               s.a3 * (l2(q + 3 * b) - l2(q - 3 * b));
    }
    __device__ __forceinline__ uint32_t full_centre(uint32_t slot) const {
        return slot + 4 * ((lz + 3) * (FY * FX) + (ly + 3) * FX + (lx + 4));
    }

    __device__ __forceinline__ void grad(int a, f2& gx, f2& gy, f2& gz) const {
        const int j = S::sten(full_seq(a));
        const uint32_t q = full_centre(R.wait_box(j));
        f2 p1, p2, p3, m1, m2, m3;
        xpairs(q, p1, p2, p3, m1, m2, m3);
        gx = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
        gy = d1(q, FX);
        gz = d1(q, FX * FY);
        R.release(j, gx.v.x + gy.v.y + gz.v.x);
    }
    __device__ __forceinline__ void grad_lap(int a, f2& gx, f2& gy, f2& gz, f2& lap) const {
        const int j = S::sten(full_seq(a));
        const uint32_t q = full_centre(R.wait_box(j));
        f2 s1, s2, s3;
        {
            f2 p1, p2, p3, m1, m2, m3;
            xpairs(q, p1, p2, p3, m1, m2, m3);
            gx = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            s1 = p1 + m1;
            s2 = p2 + m2;
            s3 = p3 + m3;
        }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
            const int b = 4 * (ax == 0 ? FX : FX * FY);
            const f2 p1 = l2(q + b), p2 = l2(q + 2 * b), p3 = l2(q + 3 * b);
            const f2 m1 = l2(q - b), m2 = l2(q - 2 * b), m3 = l2(q - 3 * b);
            const f2 g = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            if (ax == 0)
                gy = g;
            else
                gz = g;
            s1 += p1 + m1;
            s2 += p2 + m2;
            s3 += p3 + m3;
        }
        const f2 centre = l2(q);
        lap = s.l0 * centre + s.l1 * s1 + s.l2 * s2 + s.l3 * s3;
        R.release(j, lap.v.x + gx.v.y + gy.v.x + gz.v.y);
    }
    // dx(a) + dy(a+1) + dz(a+2) for a = 24, 27, 30, 33 (boxes a-24 .. a-22)
    __device__ __forceinline__ f2 div3(int a) const {
        const int jx = S::sten(a - 24), jy = S::sten(a - 23), jz = S::sten(a - 22);
        f2 dxv;
        {
            const uint32_t q = R.wait_box(jx) + 4 * (lz * (BY * FX) + ly * FX + (lx + 4));
            f2 p1, p2, p3, m1, m2, m3;
            xpairs(q, p1, p2, p3, m1, m2, m3);
            dxv = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
        }
        R.release(jx, dxv.v.x + dxv.v.y);
        const f2 dyv = d1(R.wait_box(jy) + 4 * (lz * (FY * BX) + (ly + 3) * BX + lx), BX);
        R.release(jy, dyv.v.x + dyv.v.y);
        const f2 dzv = d1(R.wait_box(jz) + 4 * ((lz + 3) * (BY * BX) + ly * BX + lx), BY * BX);
        R.release(jz, dzv.v.x + dzv.v.y);
        return dxv + dyv + dzv;
    }
};

// ------------------------------------------------------------- epilogue
struct TmaBufs {
    float* yhi;
    float* ylo;
    float* kacc;
};

// Stage 1 writes k1 and X2 = y_hi + k1 dt/2 (X1 = y_hi, the centres); stages
// 2-4 read their operands (kacc, y_hi, y_lo at the tile's sites) from global
// memory (NB = 0) or from the epilogue boxes of the ring (NB > 0).
template <int STAGE, class C, int NB>
struct TmaSink {
    using S = Seq<NB>;
    const TmaAcc<C, NB>& A;
    const Layout& L;
    TmaBufs b;
    float* __restrict__ xn;
    f2 h, w6;
    mutable uint32_t box[3];  // slots of the current epilogue group, per buffer
    __device__ __forceinline__ static float2* at(float* base, int64_t q) { return reinterpret_cast<float2*>(base + q); }
    __device__ __forceinline__ void operator()(int a, f2 r) const {
        const int64_t q = a * L.P + A.c;
        if (STAGE == 1) {
            *at(b.kacc, q) = r.v;
            *at(xn, q) = (A.v(a) + h * r).v;
            return;
        }
        if (NB == 0) {
            // read then written by this thread only: read-only path is safe
            const float2* k0 = reinterpret_cast<const float2*>(b.kacc + q);
            const float2* y0 = reinterpret_cast<const float2*>(b.yhi + q);
            if (STAGE < 4) {
                *at(b.kacc, q) = (f2(__ldg(k0)) + f2(2.f) * r).v;
                *at(xn, q) = (f2(__ldg(y0)) + h * r).v;
            } else {
                const f2 s = f2(__ldg(k0)) + r;
                f2 hi(__ldg(y0)), lo(__ldg(reinterpret_cast<const float2*>(b.ylo + q)));
                acc_hilo(hi, lo, f2(w6 * s));
                *at(b.yhi, q) = hi.v;
                *at(b.ylo, q) = lo.v;
            }
            return;
        }
        const int g = group_of(a), a0 = group_first(g);
        if (a == a0)
#pragma unroll
            for (int u = 0; u < NB; ++u) box[u] = A.R.wait_box(S::epi(g, u));
        const uint32_t off = 4 * ((((a - a0) * C::BZ + A.lz) * C::BY + A.ly) * BX + A.lx);
        float dep;
        if (STAGE < 4) {
            const f2 k = f2(lds2(box[0] + off)) + f2(2.f) * r;
            const f2 x = f2(lds2(box[1] + off)) + h * r;
            *at(b.kacc, q) = k.v;
            *at(xn, q) = x.v;
            dep = k.v.x + x.v.y;
        } else {
            const f2 s = f2(lds2(box[0] + off)) + r;
            f2 hi(lds2(box[1] + off)), lo(lds2(box[2] + off));
            acc_hilo(hi, lo, f2(w6 * s));
            *at(b.yhi, q) = hi.v;
            *at(b.ylo, q) = lo.v;
            dep = hi.v.x + lo.v.y;
        }
        if (a == a0 + group_size(g) - 1)
#pragma unroll
            for (int u = 0; u < NB; ++u) A.R.release(S::epi(g, u), dep);
    }
};

template <int STAGE, bool BETA, int TBY, int TBZ>
__global__ void __launch_bounds__(Cfg<TBY, TBZ>::NTHREADS, 1)
    k_stage_tma(const __grid_constant__ Grid g, const __grid_constant__ Layout L, const __grid_constant__ TmaMaps M,
                const __grid_constant__ EpiMaps E, const float* __restrict__ X, TmaBufs b,
                float* __restrict__ xn, PhysCoef<f2> pc, StencilCoef<f2> sc, f2 h, f2 w6, int* err, long spin) {
    using C = Cfg<TBY, TBZ>;
    constexpr int NB = !kEpilogueInRing || STAGE == 1 ? 0 : STAGE == 4 ? 3 : 2;
    constexpr int BY = C::BY, BZ = C::BZ;
    extern __shared__ __align__(128) float smem_f[];
    __shared__ __align__(8) uint64_t bars[2 * NS];
    const int tid = threadIdx.x;
    Ring<C, NB> R;
    const uint32_t pad = ((128u - (smem_u32(smem_f) & 127u)) & 127u) / 4u;  // floats to a 128-byte boundary
    R.slots = smem_u32(smem_f + pad);
    R.bars = smem_u32(bars);
    R.maps = &M;
    R.emaps = &E;
    R.err = err;
    R.spin = spin;
    R.ntx = g.nx / BX;
    R.nty = g.ny / BY;
    R.ntiles = R.ntx * R.nty * (g.nz / BZ);
    R.ok = 1;
    if ((int)blockIdx.x >= R.ntiles) return;
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(R.full(s), 1);
            mbar_init(R.empty(s), C::NWARP);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (tid >= C::NT) {  // the producer warp
        if (tid == C::NT) R.produce();
        return;
    }
    const int lx = 2 * (tid % (BX / 2)), ly = (tid / (BX / 2)) % BY, lz = tid / ((BX / 2) * BY);
    for (int t = blockIdx.x, it = 0; t < R.ntiles; t += gridDim.x, ++it) {
        R.set_tile(t, it);
        const int i0 = R.x0 + lx, j = R.y0 + ly, k = R.z0 + lz;
        TmaAcc<C, NB> A{R, X, L.P, (int)L.at(i0, j, k), lx, ly, lz, sc};
        TmaSink<STAGE, C, NB> out{A, L, b, xn, h, w6, {0u, 0u, 0u}};
        site_rates<f2, BETA>(A, pc, out);
    }
}

// ------------------------------------------------------------- host side
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    return fn;
}

// tile boxes of n arrays (epilogue operands)
bool encode_tile(CUtensorMap* M, float* base, const Layout& L, int BY, int BZ, int n) {
    EncodeFn enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)L.px, (cuuint64_t)L.py, (cuuint64_t)L.pz, 36};
    const cuuint64_t strides[3] = {(cuuint64_t)L.px * 4, (cuuint64_t)L.px * L.py * 4, (cuuint64_t)L.P * 4};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const cuuint32_t box[4] = {BX, (cuuint32_t)BY, (cuuint32_t)BZ, (cuuint32_t)n};
    return enc(M, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_maps(TmaMaps* M, float* base, const Layout& L, int BY, int BZ) {
    const int FY = BY + 6, FZ = BZ + 6;
    EncodeFn enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)L.px, (cuuint64_t)L.py, (cuuint64_t)L.pz, 36};
    const cuuint64_t strides[3] = {(cuuint64_t)L.px * 4, (cuuint64_t)L.px * L.py * 4, (cuuint64_t)L.P * 4};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const cuuint32_t bx = BX, fx = FX, by = BY, bz = BZ, fy = FY, fz = FZ;
    const cuuint32_t boxes[4][4] = {{fx, by, bz, 1}, {bx, fy, bz, 1}, {bx, by, fz, 1}, {fx, fy, fz, 1}};
    for (int q = 0; q < 4; ++q)
        if (enc(&M->m[q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, boxes[q], es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    return true;
}

// per-context state: tile shape, maps of the three stencil sources, error word, grid
struct TmaState {
    int by = 0, bz = 0;
    TmaMaps yhi, xa, xb;
    EpiMaps epi;  // [kacc, yhi, ylo]
    int* err = nullptr;
    int grid = 0;
    long spin = kSpin;  // wait limit in polls (ewpt_set_wait_limit)
};

template <bool BETA, int TBY, int TBZ>
void step_tma(const Grid& g, const Layout& L, const TmaState& T, TmaBufs b, float* xa, float* xb,
              const PhysCoef<f2>& pc, const StencilCoef<f2>& sc, double dt, cudaStream_t st) {
    using C = Cfg<TBY, TBZ>;
    const f2 h2((float)(dt / 2.)), h1((float)dt), w6((float)(dt / 6.)), z(0.f);
    const int G = T.grid, n = C::NTHREADS, sm = C::SMEM_BYTES;
    k_stage_tma<1, BETA, TBY, TBZ><<<G, n, sm, st>>>(g, L, T.yhi, T.epi, b.yhi, b, xa, pc, sc, h2, w6, T.err, T.spin);
    launch_ghost_fill(g, L, xa, st, true);
    k_stage_tma<2, BETA, TBY, TBZ><<<G, n, sm, st>>>(g, L, T.xa, T.epi, xa, b, xb, pc, sc, h2, w6, T.err, T.spin);
    launch_ghost_fill(g, L, xb, st, true);
    k_stage_tma<3, BETA, TBY, TBZ><<<G, n, sm, st>>>(g, L, T.xb, T.epi, xb, b, xa, pc, sc, h1, w6, T.err, T.spin);
    launch_ghost_fill(g, L, xa, st, true);
    k_stage_tma<4, BETA, TBY, TBZ><<<G, n, sm, st>>>(g, L, T.xa, T.epi, xa, b, nullptr, pc, sc, z, w6, T.err, T.spin);
    launch_ghost_fill(g, L, b.yhi, st, true);
}

template <int TBY, int TBZ>
cudaError_t setup_variant(int* per_sm) {
    using C = Cfg<TBY, TBZ>;
    const int sm = C::SMEM_BYTES;
    const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(k_stage_tma<1, false, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<2, false, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<3, false, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<4, false, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<1, true, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<2, true, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<3, true, TBY, TBZ>, A, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stage_tma<4, true, TBY, TBZ>, A, sm);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_stage_tma<2, false, TBY, TBZ>, C::NTHREADS,
                                                          sm);
    return e;
}

bool shape_ok(int by, int bz) { return bz == 4 && (by == 2 || by == 4); }

}  // namespace

bool tma_tiling_fits(const Grid& g, int by, int bz) {
    return shape_ok(by, bz) && g.nx % BX == 0 && g.ny % by == 0 && g.nz % bz == 0;
}

void ewpt_tma_release(ewpt_ctx* c) {
    TmaState* T = static_cast<TmaState*>(c->tma);
    if (!T) return;
    cudaFree(T->err);
    delete T;
    c->tma = nullptr;
}

// Encode the tensor maps for tiles of 32 x by x bz sites and size the
// persistent grid (again whenever the tile shape changes).
int ewpt_tma_prepare(ewpt_ctx* c, int by, int bz) {
    if (c->p.precision != EWPT_FP32 || c->lay.gx == 0)
        return ewpt_fail(c, EWPT_ERR_STATE, "TMA tiles need the FP32 form");
    if (!shape_ok(by, bz)) return ewpt_fail(c, EWPT_ERR_ARG, "TMA tiles: 32 x {2,4} x 4 sites");
    if (!tma_tiling_fits(c->g, by, bz))
        return ewpt_fail(c, EWPT_ERR_ARG, "TMA tiles need nx %% %d == 0, ny %% %d == 0, nz %% %d == 0", BX, by, bz);
    TmaState* T = static_cast<TmaState*>(c->tma);
    if (T && T->by == by && T->bz == bz) return EWPT_OK;
    TmaMaps m[3];
    EpiMaps em;
    const int ld = c->lay.lead;
    bool okm = encode_maps(&m[0], c->y32.hi + ld, c->lay, by, bz) && encode_maps(&m[1], c->w32.xa + ld, c->lay, by, bz) &&
               encode_maps(&m[2], c->w32.xb + ld, c->lay, by, bz);
    float* eb[3] = {c->w32.kacc, c->y32.hi, c->y32.lo};
    for (int q = 0; q < 3 && okm; ++q)
        okm = encode_tile(&em.m[q][0], eb[q] + ld, c->lay, by, bz, 8) && encode_tile(&em.m[q][1], eb[q] + ld, c->lay, by, bz, 1);
    if (!okm) return ewpt_fail(c, EWPT_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    int per_sm = 0, nsm = 0;
    cudaError_t e = by == 4 ? setup_variant<4, 4>(&per_sm) : setup_variant<2, 4>(&per_sm);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->p.device);
    if (e != cudaSuccess || per_sm < 1)
        return ewpt_fail(c, EWPT_ERR_CUDA, "TMA stage kernel setup: %s",
                         e != cudaSuccess ? cudaGetErrorString(e) : "no resident block");
    if (!T) {
        T = new TmaState();
        e = cudaMalloc(&T->err, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(T->err, 0, sizeof(int));
        if (e != cudaSuccess) {
            cudaFree(T->err);
            delete T;
            return ewpt_cuda_check(c, e, "TMA error word");
        }
        c->tma = T;
    }
    T->by = by;
    T->bz = bz;
    T->yhi = m[0];
    T->xa = m[1];
    T->xb = m[2];
    T->epi = em;
    ewpt_tma_set_spin(c);
    const int ntiles = (c->g.nx / BX) * (c->g.ny / by) * (c->g.nz / bz);
    T->grid = std::min(ntiles, per_sm * nsm);
    return EWPT_OK;
}

// Wait limit of the TMA stage kernels' mbarrier waits, in polls (< 0: the
// default kSpin); kept in the context and applied to its TMA state.
void ewpt_tma_set_spin(ewpt_ctx* c) {
    TmaState* T = static_cast<TmaState*>(c->tma);
    if (T) T->spin = c->wait_polls < 0 ? kSpin : (long)c->wait_polls;
}

// Read and clear the error word of the TMA stage kernels (synchronous).
int ewpt_tma_check(ewpt_ctx* c) {
    TmaState* T = static_cast<TmaState*>(c->tma);
    if (!T) return EWPT_OK;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, T->err, sizeof(int), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) return ewpt_cuda_check(c, e, "TMA error word");
    if (h) {
        cudaMemsetAsync(T->err, 0, sizeof(int), c->st);
        return ewpt_fail(c, EWPT_ERR_TIMEOUT, "a TMA pipeline wait in the stage kernel ran out (results invalid)");
    }
    return EWPT_OK;
}

cudaError_t launch_step_fp32_tma(ewpt_ctx* c, double Jex, double gam) {
    const TmaState* T = static_cast<const TmaState*>(c->tma);
    if (!T) return cudaErrorInvalidValue;
    const PhysCoef<f2> pc = make_phys<f2>(c->p, Jex, gam);
    const StencilCoef<f2> sc = pair_stencil(make_stencil<float>(c->p.dx));
    TmaBufs b{c->y32.hi, c->y32.lo, c->w32.kacc};
    const bool beta = c->p.beta_w != 0.0 || c->p.beta_y != 0.0;
    if (T->by == 4) {
        if (beta)
            step_tma<true, 4, 4>(c->g, c->lay, *T, b, c->w32.xa, c->w32.xb, pc, sc, c->p.dt, c->st);
        else
            step_tma<false, 4, 4>(c->g, c->lay, *T, b, c->w32.xa, c->w32.xb, pc, sc, c->p.dt, c->st);
    } else {
        if (beta)
            step_tma<true, 2, 4>(c->g, c->lay, *T, b, c->w32.xa, c->w32.xb, pc, sc, c->p.dt, c->st);
        else
            step_tma<false, 2, 4>(c->g, c->lay, *T, b, c->w32.xa, c->w32.xb, pc, sc, c->p.dt, c->st);
    }
    return cudaGetLastError();
}
