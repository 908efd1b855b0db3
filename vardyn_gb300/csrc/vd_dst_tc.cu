// x-direction DST-I pass on the 5th-generation tensor cores (tcgen05, sm_103a)
// for float32 plans.
//
// The pass is two dense half-size products per row block (even/odd split, see
// vd_dst.cu). Each CTA owns 128 interior rows (UMMA M = 128) and a group of
// consecutive 32-column output tiles (up to 256 columns forward, 128 per
// parity inverse) held in tensor memory (TMEM, fp32 accumulators). The group
// size is chosen per launch so that small batches still fill the GPU: the B
// operand of a group is the concatenation of its tiles' pre-swizzled images,
// because a 32-row slab of the 128B-swizzled K-major layout is exactly the
// next 4 KB of the tile.
// Float32 accuracy comes from the 3xTF32 split: x = x_hi + x_lo with
// x_hi = tf32(x), and x.w ~= x_hi.w_hi + x_hi.w_lo + x_lo.w_hi (the dropped
// x_lo.w_lo term is ~2^-22 relative).
//
// Pipeline (per K chunk of 32 = one 128-byte swizzle row of fp32):
//   warps 0-15 build the A chunk (butterfly or copy of the input rows, hi/lo
//              split; 8 rows each) in the 128B-swizzled K-major layout and
//              arrive on fullA;
//   thread 0   also issues the bulk copies (cp.async.bulk) of the
//              pre-swizzled hi/lo chunks of the DST half matrix (fullB);
//   warp 16    owns the TMEM allocation; its lane 0 issues 3 x 4 MMAs per
//              chunk and commits to `empty` to recycle the stage;
//   warps 0-15 finally read the accumulators (tcgen05.ld) and write rows;
//              in the inverse pass the two CTAs of a cluster (odd-k and
//              even-k sums) first swap half tiles with one bulk copy each.
// Every mbarrier wait is bounded (2 s of %globaltimer); a timeout sets a bit
// in a device flag (vd_device_error) and the CTA finishes without hanging.
#include "vd_internal.cuh"
#include <algorithm>
#include <vector>
#include <cmath>
#include <cstring>
#include <mutex>

namespace vd {

__device__ int g_tc_error = 0;

namespace tc {

constexpr int BM = 128;
constexpr int KCH = 32;
constexpr int NPW = 16;                // producer / epilogue warps
constexpr int RPW = 128 / NPW;         // A rows per producer warp
constexpr int NPROD = NPW * 32;
constexpr int NTHREADS = NPROD + 32;   // + warp NPW: TMEM owner and MMA issuer
constexpr int MAX_STAGES = 6;
constexpr int TMEM_COLS = 256;
constexpr int TILE = 32;                           // columns of one B image tile
constexpr uint32_t TILE_BYTES = TILE * 32 * 4;     // 4 KB: 32 rows of the swizzled layout
constexpr uint32_t A_TILE = BM * KCH * 4;          // 16 KB
constexpr size_t PIPE_BYTES = 200 * 1024;          // pipeline stages fit in this
constexpr int EPI_S = 257;                          // row pitch of the epilogue staging tile
constexpr size_t EPI_BYTES = (size_t)BM * EPI_S * 4; // epilogue staging tile (reuses the stages)
// inverse pass: half of the peer CTA's staging tile, received after ours
constexpr uint32_t HALF_ROWS = BM / 2;
constexpr uint32_t HALF_BYTES = HALF_ROWS * EPI_S * 4;
constexpr size_t SMEM_MAX = PIPE_BYTES + 1024;      // largest dynamic request of any launch

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on the phase of parity `parity`.
// The timer is read once every 64 polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 0 && gtimer() - t0 > 2000000000ull) {
            atomicOr(&g_tc_error, code);
            return false;
        }
    }
}

// Distributed shared memory of a 2-CTA cluster (the inverse pass).
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
// Every thread of both CTAs arrives; shared-memory writes before the
// barrier are visible to the peer CTA after it.
__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Shared memory of this CTA -> shared memory of a CTA of the cluster; the
// bytes complete on `bar`, a barrier of the destination CTA.
__device__ __forceinline__ void bulk_s2s_cluster(uint32_t dst, uint32_t src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "r"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) | ((uint64_t)(1024u >> 4) << 32) |
           ((uint64_t)1u << 46) | ((uint64_t)2u << 61);
}

// Instruction descriptor of kind::tf32: fp32 accumulate, tf32 A and B, both
// K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of fp32 element (r, k) in a [rows][32] 128B-swizzled tile
__host__ __device__ constexpr uint32_t swz(int r, int k)
{
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 2) ^ (r & 7)) & 7) << 4) + (k & 3) * 4);
}

}  // namespace tc

constexpr int MAX_TILES = 64;   // ne <= 2048

// Images: per parity (forward) or job (inverse), per K chunk, the hi then the
// lo part of the whole [Ntot][32] swizzled operand, so that the rows of any
// run of consecutive 32-row tiles are one contiguous range.
struct TcTab {
    int kch;                         // K chunks of 32
    int nt;                          // 32-column tiles over the ne output columns
    int Ntot;                        // operand rows: 32*(nt-1) + last tile (a multiple of 16)
    long long fwd_base[2];           // forward image offsets (floats) per parity
    long long inv_base[2];           // inverse image offsets (floats) per job
    int gf, gi;                      // tiles per CTA of this launch (forward <= 8, inverse <= 4)
    int nst;                         // pipeline stages of this launch (<= MAX_STAGES)
    uint32_t b_tile;                 // bytes of one B operand (hi or lo) in a stage
};

struct TcGeom {
    int n, ne, no, my, nx;
    long long fs;
    int R, lds;
};

using namespace tc;

template <int MODE, int EPI>
__global__ void __launch_bounds__(NTHREADS, 1)
dst_tc_kernel(TcGeom g, TcTab tab, const float* __restrict__ img, const float* __restrict__ src,
              const float* __restrict__ sub, int sub_batches, float* __restrict__ spec, float* __restrict__ out,
              const float* __restrict__ add, int add_batches, const int8_t* __restrict__ mask)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[3 * MAX_STAGES + 2];
    __shared__ uint32_t tmem_base_sh;
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_u32(sm);
    // stage s: A hi | A lo | B hi | B lo (every part 1024-byte aligned)
    const int STAGES = tab.nst;
    const uint32_t stage_bytes = 2 * A_TILE + 2 * tab.b_tile;
    auto a_hi = [&](int s) { return sbase + s * stage_bytes; };
    auto a_lo = [&](int s) { return sbase + s * stage_bytes + A_TILE; };
    auto b_hi = [&](int s) { return sbase + s * stage_bytes + 2 * A_TILE; };
    auto b_lo = [&](int s) { return sbase + s * stage_bytes + 2 * A_TILE + tab.b_tile; };
    const uint32_t bar0 = smem_u32(&bars[0]);
    auto fullA = [&](int s) { return bar0 + 8u * s; };
    auto fullB = [&](int s) { return bar0 + 8u * (STAGES + s); };
    auto empty = [&](int s) { return bar0 + 8u * (2 * STAGES + s); };
    const uint32_t accf = bar0 + 8u * (3 * STAGES);
    const uint32_t rbar = bar0 + 8u * (3 * STAGES + 1);   // inverse: the peer's half tile has landed

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;

    // ---- job layout of this CTA --------------------------------------------
    // Forward: tiles [t_first, t_first + ntl) of one output parity. Inverse:
    // the CTA pair of a cluster shares the rows and the tiles; rank 0 takes
    // the odd-k rows of the spectrum (job 0), rank 1 the even-k rows (job 1),
    // and the epilogue exchanges half tiles with one bulk copy into the
    // peer's shared memory (distributed shared memory).
    int half = 0, t_first, ntl, cjob = 0;
    if (MODE == 0) {
        const int G = (tab.nt + tab.gf - 1) / tab.gf;
        half = blockIdx.x / G;
        t_first = (blockIdx.x - half * G) * tab.gf;
        ntl = min(tab.gf, tab.nt - t_first);
    } else {
        cjob = blockIdx.x & 1;
        t_first = (blockIdx.x >> 1) * tab.gi;
        ntl = min(tab.gi, tab.nt - t_first);
    }
    const int njobs = 1;
    const int N = min(TILE * ntl, tab.Ntot - TILE * t_first);
    const int nchunks = njobs * tab.kch;
    const uint32_t b_bytes = (uint32_t)N * KCH * 4;

    constexpr int MMA_WARP = NPROD / 32;
    if (warp == MMA_WARP) {
        tmem_alloc(smem_u32(&tmem_base_sh), TMEM_COLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(fullA(s), NPROD);
            mbar_init(fullB(s), 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(accf, 1);
        if (MODE == 1) mbar_init(rbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // armed before the cluster barrier after which the peer sends
        if (MODE == 1) mbar_arrive_expect_tx(rbar, HALF_BYTES);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;

    const int n = g.n, ne = g.ne, no = g.no;
    if (warp < MMA_WARP) {
        // ------------------------------ producers ------------------------------
        // warp w fills rows [RPW w, RPW (w+1)) of the A chunk; lane l handles K
        // index k0 + l, so every global load is one coalesced 128-byte row.
        // The element offsets of the warp's 16 rows do not change from chunk
        // to chunk: they are computed once (32-bit; the host checks that the
        // arrays are smaller than 2^31 elements). Rows past the end repeat
        // the last valid row and are zeroed when the chunk is stored.
        const int r0 = warp * RPW;
        const int row0 = blockIdx.y * BM + r0;
        int roff[RPW];
        uint32_t rvalid = 0;
        {
            int f = 0, j = 1;
            if (MODE == 0) {
                const int rr = min(row0, g.R - 1);
                f = rr / g.my;
                j = rr - f * g.my + 1;
            }
            int last = 0;
#pragma unroll
            for (int i = 0; i < RPW; ++i) {
                const int row = row0 + i;
                const bool v = row < g.R;
                int o;
                if (MODE == 0) {
                    o = f * (int)g.fs + j * g.nx + 1;
                    if (v && ++j > g.my) {
                        j = 1;
                        ++f;
                    }
                } else {
                    o = row * g.lds;
                }
                if (v) {
                    last = o;
                    rvalid |= 1u << i;
                }
                roff[i] = v ? o : last;
            }
        }
        const bool use_sub = (MODE == 0) && sub != nullptr;
        const float* __restrict__ base_ptr = (MODE == 0) ? src : spec;
        // Two register buffers: the loads of chunk c+2 are issued right after
        // chunk c is stored, so their latency overlaps the processing of
        // chunk c+1, the wait for a free stage and the MMAs.
        auto load_chunk = [&](int c, float (&x1)[RPW], float (&x2)[RPW]) {
            const int job = cjob;
            const int kc = c;
            const int p = kc * KCH + lane;
            int lim, c1, c2;
            if (MODE == 0) {
                lim = half == 0 ? ne : no;
                c1 = p;
                c2 = n - 1 - p;
            } else {
                lim = job == 0 ? ne : no;
                c1 = job == 0 ? p : ne + p;
                c2 = 0;
            }
            const bool pv = p < lim;
            const int cc1 = pv ? c1 : 0;
            const int cc2 = (pv && p < no) ? c2 : 0;
            const float* __restrict__ b1 = base_ptr + cc1;
            const float* __restrict__ b2 = base_ptr + cc2;
            if (MODE == 0 && use_sub) {
                // nonzero background PV: subtract it (rare path)
                const float* __restrict__ s1 = sub + cc1;
                const float* __restrict__ s2 = sub + cc2;
#pragma unroll
                for (int i = 0; i < RPW; ++i) {
                    const bool hs = roff[i] < sub_batches * (int)g.fs;
                    x1[i] = __ldg(b1 + roff[i]) - (hs ? __ldg(s1 + roff[i]) : 0.f);
                    x2[i] = __ldg(b2 + roff[i]) - (hs ? __ldg(s2 + roff[i]) : 0.f);
                }
                return;
            }
#pragma unroll
            for (int i = 0; i < RPW; ++i) {
                x1[i] = __ldg(b1 + roff[i]);
                if (MODE == 0) x2[i] = __ldg(b2 + roff[i]);
            }
        };
        // shared-memory byte offset of (row r0 + i, k = lane) in a swizzled
        // [128][32] fp32 tile: r0 is a multiple of 8, so only i enters the
        // XOR pattern (a compile-time constant per unrolled i)
        const uint32_t sw_row = (uint32_t)(r0 >> 3) * 1024u + (uint32_t)(lane & 3) * 4u;
        const uint32_t sw_q = (uint32_t)(lane >> 2);
        // stage / phase of the next chunk to store (chunks are stored in order)
        int ps = 0;
        uint32_t pu = 0;
        auto process = [&](int c, const float (&x1)[RPW], const float (&x2)[RPW]) {
            const int s = ps;
            const uint32_t u = pu;
            if (++ps == STAGES) {
                ps = 0;
                ++pu;
            }
            const int job = cjob;
            const int kc = c;
            if (c >= STAGES) mbar_wait(empty(s), (u - 1) & 1, 1);
            if (tid == 0) {
                mbar_arrive_expect_tx(fullB(s), 2 * b_bytes);
                const long long base = MODE == 0 ? (half ? tab.fwd_base[1] : tab.fwd_base[0])
                                                 : (job ? tab.inv_base[1] : tab.inv_base[0]);
                const float* blk = img + base + (size_t)kc * 2 * tab.Ntot * KCH + (size_t)t_first * TILE * KCH;
                bulk_g2s(b_hi(s), blk, b_bytes, fullB(s));
                bulk_g2s(b_lo(s), blk + (size_t)tab.Ntot * KCH, b_bytes, fullB(s));
            }
            const int p = kc * KCH + lane;
            const bool p2 = p < no;
            const int limv = (MODE == 0) ? (half == 0 ? ne : no) : (job == 0 ? ne : no);
            const uint32_t keep = (p < limv) ? rvalid : 0u;
            const uint32_t ah = a_hi(s) + sw_row, al = a_lo(s) + sw_row;
#pragma unroll
            for (int i = 0; i < RPW; ++i) {
                float val;
                if (MODE == 0)
                    val = p2 ? (half == 0 ? x1[i] + x2[i] : x1[i] - x2[i]) : x1[i];
                else
                    val = x1[i];
                val = ((keep >> i) & 1u) ? val : 0.f;
                const float h = tf32_rna(val);
                const float l = tf32_rna(val - h);
                const uint32_t off = (uint32_t)(i >> 3) * 1024u + (uint32_t)(i & 7) * 128u +
                                     (((sw_q ^ (uint32_t)(i & 7)) & 7u) << 4);
                asm volatile("st.shared.f32 [%0], %1;" ::"r"(ah + off), "f"(h) : "memory");
                asm volatile("st.shared.f32 [%0], %1;" ::"r"(al + off), "f"(l) : "memory");
            }
            fence_async_smem();
            mbar_arrive(fullA(s));
        };
        float xa1[RPW], xa2[RPW], xb1[RPW], xb2[RPW];
        load_chunk(0, xa1, xa2);
        if (nchunks > 1) load_chunk(1, xb1, xb2);
        for (int c = 0; c < nchunks; c += 2) {
            process(c, xa1, xa2);
            if (c + 2 < nchunks) load_chunk(c + 2, xa1, xa2);
            if (c + 1 < nchunks) {
                process(c + 1, xb1, xb2);
                if (c + 3 < nchunks) load_chunk(c + 3, xb1, xb2);
            }
        }

        // ------------------------------ epilogue -------------------------------
        // accumulators -> shared staging tile [128][S], then coalesced row
        // stores. Warps w, w+4, w+8, w+12 share TMEM lanes 32(w%4).. and split
        // the columns. All stages are free once the last MMA has completed.
        mbar_wait(accf, 0, 4);
        tc_fence_after();
        constexpr int S = EPI_S;
        float* ep = reinterpret_cast<float*>(sm);
        const int sp = warp & 3;
        const int hc = warp >> 2;
        const int trow = sp * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(sp * 32) << 16);
        constexpr int NQ = NPW / 4;     // warps per TMEM lane quarter
        const int per = (((N + NQ - 1) / NQ + 31) / 32) * 32;
        const int cbeg = min(N, hc * per);
        const int cend = min(N, cbeg + per);
        for (int cg = cbeg; cg < cend; cg += 32) {
            float vv[32];
            tmem_ld32(lane_base + cg, vv);
#pragma unroll
            for (int i = 0; i < 32; ++i) ep[trow * S + cg + i] = vv[i];
        }
        if (MODE == 0) {
            asm volatile("bar.sync 1, %0;" ::"n"(NPROD) : "memory");
            const int lim = half == 0 ? ne : no;
            const int coff = half == 0 ? 0 : ne;
            const int t0 = t_first * TILE;
            for (int rr = 0; rr < RPW; ++rr) {
                const int r = r0 + rr;
                const int row = blockIdx.y * BM + r;
                if (row >= g.R) break;
                float* drow = spec + (long long)row * g.lds + coff;
                for (int cc = lane; cc < N; cc += 32) {
                    const int t = t0 + cc;
                    if (t < lim) drow[t] = ep[r * S + cc];
                }
            }
        }
    } else if (lane == 0) {
        // ------------------------------ MMA issuer -----------------------------
        const uint32_t idesc = idesc_tf32(BM, N);
        int s = 0;
        uint32_t u = 0;
        for (int c = 0; c < nchunks; ++c) {
            const int kc = c;
            mbar_wait(fullA(s), u & 1, 2);
            mbar_wait(fullB(s), u & 1, 2);
            tc_fence_after();
            const uint32_t d = tmem;
#pragma unroll
            for (int kk = 0; kk < KCH / 8; ++kk) {
                const uint64_t ah = sdesc_sw128(a_hi(s) + kk * 32);
                const uint64_t al = sdesc_sw128(a_lo(s) + kk * 32);
                const uint64_t bh = sdesc_sw128(b_hi(s) + kk * 32);
                const uint64_t bl = sdesc_sw128(b_lo(s) + kk * 32);
                mma_tf32(d, ah, bh, idesc, (kc > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(d, ah, bl, idesc, 1u);
                mma_tf32(d, al, bh, idesc, 1u);
            }
            mma_commit(empty(s));
            if (++s == STAGES) {
                s = 0;
                ++u;
            }
        }
        mma_commit(accf);
    }
    __syncwarp();
    if constexpr (MODE == 1) {
        // ---------------- inverse epilogue across the CTA pair ----------------
        // Rank 0 holds the odd-k sums A, rank 1 the even-k sums B of all 128
        // rows. Each CTA sends the half of its staging tile that the peer
        // needs with one bulk copy into the peer's free pipeline space (rank
        // 0 its rows 64..127, rank 1 its rows 0..63), then combines its own
        // 64 rows locally: x[p] = A + B and x[n-1-p] = A - B. Every thread of
        // both CTAs reaches both cluster barriers.
        constexpr int S = EPI_S;
        const uint32_t recv = smem_u32(sm) + (uint32_t)EPI_BYTES;
        if (warp < MMA_WARP) fence_async_smem();   // staging writes -> the copy
        cluster_sync_all();
        if (tid == 0) {
            const uint32_t src = smem_u32(sm) + (cjob == 0 ? HALF_BYTES : 0u);
            bulk_s2s_cluster(mapa_shared(recv, (uint32_t)(cjob ^ 1)), src, HALF_BYTES,
                             mapa_shared(rbar, (uint32_t)(cjob ^ 1)));
        }
        if (warp < MMA_WARP && mbar_wait(rbar, 0, 16)) {
            const float* ep = reinterpret_cast<const float*>(sm);
            const float* pe = reinterpret_cast<const float*>(sm + EPI_BYTES);
            constexpr int RW = (int)HALF_ROWS / NPW;    // rows per warp
            const int p0 = t_first * TILE;
            for (int rr = 0; rr < RW; ++rr) {
                const int rl = warp * RW + rr;              // row in the received half
                const int r = (int)(cjob * HALF_ROWS) + rl; // row in the 128-row block
                const int row = blockIdx.y * BM + r;
                if (row >= g.R) break;
                const int f = row / g.my;
                const int j = row - f * g.my + 1;
                const long long base = f * g.fs + (long long)j * g.nx + 1;
                const bool ha = add != nullptr && (EPI != EPI_H || f < add_batches);
                float va[8], vb[8], a1[8], a2[8];
                bool m1[8], m2[8];
                // every load of the row first, then the stores
#pragma unroll
                for (int u8 = 0; u8 < 8; ++u8) {
                    const int cc = lane + 32 * u8;
                    const int p = p0 + cc;
                    const bool v1 = cc < N && p < ne, v2 = cc < N && p < no;
                    const float own = cc < N ? ep[r * S + cc] : 0.f;
                    const float oth = cc < N ? pe[rl * S + cc] : 0.f;
                    va[u8] = cjob == 0 ? own : oth;
                    vb[u8] = cjob == 0 ? oth : own;
                    const int c1 = p, c2 = n - 1 - p;
                    a1[u8] = (v1 && ha) ? add[base + c1] : 0.f;
                    a2[u8] = (v2 && ha) ? add[base + c2] : 0.f;
                    m1[u8] = (EPI == EPI_ADJQ) ? (v1 && mask[j * g.nx + 1 + c1] == 3) : v1;
                    m2[u8] = (EPI == EPI_ADJQ) ? (v2 && mask[j * g.nx + 1 + c2] == 3) : v2;
                }
#pragma unroll
                for (int u8 = 0; u8 < 8; ++u8) {
                    const int cc = lane + 32 * u8;
                    const int p = p0 + cc;
                    if (cc < N && p < ne) {
                        const float val = va[u8] + (p < no ? vb[u8] : 0.f);
                        out[base + p] = m1[u8] ? val + a1[u8] : 0.f;
                    }
                    if (cc < N && p < no) out[base + (n - 1 - p)] = m2[u8] ? (va[u8] - vb[u8]) + a2[u8] : 0.f;
                }
            }
        }
        // the peer's copy out of this CTA's tile has landed before either exits
        cluster_sync_all();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == MMA_WARP) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// Host side: pre-swizzled hi/lo images of the half matrices
// ---------------------------------------------------------------------------
static float tf32_rna_host(float x)
{
    uint32_t b;
    std::memcpy(&b, &x, 4);
    if ((b & 0x7f800000u) != 0x7f800000u) {
        b += 0x1000u;
        b &= 0xFFFFE000u;
    }
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

struct TcPlanData {
    float* img;
    TcTab tab;
};

int build_tc_images(vd_qg1l_plan* p)
{
    const DSTTables& t = p->dst;
    const int n = t.n, ne = t.ne, no = t.no;
    TcPlanData* d = new TcPlanData();
    std::memset(&d->tab, 0, sizeof(TcTab));
    TcTab& tab = d->tab;
    tab.kch = (ne + KCH - 1) / KCH;
    tab.nt = (ne + TILE - 1) / TILE;
    if (tab.nt > MAX_TILES) { delete d; return VD_ERR_UNSUPPORTED; }
    const double scale = std::sqrt(2.0 / (n + 1));
    const long long period = 2LL * (n + 1);
    auto S = [&](long long m) { m %= period; return scale * std::sin(M_PI * double(m) / double(n + 1)); };
    // B operands as [N row][K] functions
    auto fwd_odd = [&](int tt, int pp) { return (tt < ne && pp < ne) ? S((long long)(pp + 1) * (2 * tt + 1)) : 0.0; };
    auto fwd_even = [&](int tt, int pp) { return (tt < no && pp < no) ? S((long long)(pp + 1) * (2 * tt + 2)) : 0.0; };
    auto inv_odd = [&](int pp, int tt) { return (pp < ne && tt < ne) ? S((long long)(pp + 1) * (2 * tt + 1)) : 0.0; };
    auto inv_even = [&](int pp, int tt) { return (pp < no && tt < no) ? S((long long)(pp + 1) * (2 * tt + 2)) : 0.0; };

    std::vector<float> img;
    auto emit = [&](auto fn, int row0, int N) {
        const long long off = (long long)img.size();
        for (int c = 0; c < tab.kch; ++c) {
            std::vector<float> hi(size_t(N) * KCH, 0.f), lo(size_t(N) * KCH, 0.f);
            for (int r = 0; r < N; ++r)
                for (int k = 0; k < KCH; ++k) {
                    const float v = (float)fn(row0 + r, c * KCH + k);
                    const float h = tf32_rna_host(v);
                    const float l = tf32_rna_host(v - h);
                    const uint32_t o = swz(r, k) / 4;
                    hi[o] = h;
                    lo[o] = l;
                }
            img.insert(img.end(), hi.begin(), hi.end());
            img.insert(img.end(), lo.begin(), lo.end());
        }
        return off;
    };
    tab.Ntot = ((ne + 15) / 16) * 16;
    tab.fwd_base[0] = emit(fwd_odd, 0, tab.Ntot);
    tab.fwd_base[1] = emit(fwd_even, 0, tab.Ntot);
    tab.inv_base[0] = emit(inv_odd, 0, tab.Ntot);
    tab.inv_base[1] = emit(inv_even, 0, tab.Ntot);
    if (cudaMalloc(&d->img, img.size() * sizeof(float)) != cudaSuccess) { delete d; return VD_ERR_CUDA; }
    if (cudaMemcpy(d->img, img.data(), img.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d->img);
        delete d;
        return VD_ERR_CUDA;
    }
    p->dst.tc = d;
    return VD_OK;
}

void free_tc_images(vd_qg1l_plan* p)
{
    TcPlanData* d = (TcPlanData*)p->dst.tc;
    if (!d) return;
    cudaFree(d->img);
    delete d;
    p->dst.tc = nullptr;
}

static PerDeviceOnce g_tc_once;

static cudaError_t tc_configure()
{
    return g_tc_once.run([]() -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(dst_tc_kernel<0, EPI_H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)SMEM_MAX);
        if (!e) e = cudaFuncSetAttribute(dst_tc_kernel<1, EPI_H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SMEM_MAX);
        if (!e) e = cudaFuncSetAttribute(dst_tc_kernel<1, EPI_ADJQ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SMEM_MAX);
        return e;
    });
}

// The producers address rows with 32-bit element offsets.
bool tc_fits(const vd_qg1l_plan* p, int nf)
{
    const DSTTables& t = p->dst;
    const long long fs = (long long)p->d.ny * p->d.nx;
    return (long long)nf * fs < (1LL << 31) && (long long)nf * t.my * t.lds < (1LL << 31);
}

// One x-direction pass on the tensor cores (forward: fields -> spec,
// inverse: spec -> out with the epilogue of `a`).
int dst_pass_tc(const vd_qg1l_plan* p, int nf, const SolveArgs& a, float* spec, bool fwd, cudaStream_t st)
{
    const TcPlanData* d = (const TcPlanData*)p->dst.tc;
    if (!d || !tc_fits(p, nf)) return VD_ERR_UNSUPPORTED;
    if (tc_configure() != cudaSuccess) return VD_ERR_CUDA;
    const DSTTables& t = p->dst;
    TcGeom g;
    g.n = t.n; g.ne = t.ne; g.no = t.no; g.my = t.my; g.nx = p->d.nx;
    g.fs = (long long)p->d.ny * p->d.nx;
    g.R = nf * t.my;
    g.lds = t.lds;
    const int rows = (g.R + BM - 1) / BM;
    // Tiles per CTA: the widest group (fewest re-reads of the A rows) that
    // still launches ~120 CTAs on the 152 SMs.
    TcTab tab = d->tab;
    const int nt = tab.nt;
    auto groups = [&](int gsz) { return (nt + gsz - 1) / gsz; };
    tab.gf = 1;
    for (int gsz : {8, 4, 2}) {
        if (2LL * groups(gsz) * rows >= 120) { tab.gf = gsz; break; }
    }
    tab.gi = 1;
    for (int gsz : {8, 4, 2}) {
        if (2LL * groups(gsz) * rows >= 120) { tab.gi = gsz; break; }
    }
    if (p->sched.tc_group_fwd > 0) tab.gf = p->sched.tc_group_fwd;
    if (p->sched.tc_group_inv > 0) tab.gi = p->sched.tc_group_inv;
    // as many stages as the B operand size of the launch allows
    const int gmax = fwd ? tab.gf : tab.gi;
    tab.b_tile = (uint32_t)gmax * TILE_BYTES;
    const size_t stage_bytes = 2 * (size_t)A_TILE + 2 * (size_t)tab.b_tile;
    tab.nst = (int)std::min<size_t>(MAX_STAGES, PIPE_BYTES / stage_bytes);
    // the inverse also receives half of the peer's staging tile after its own
    const size_t epi = fwd ? EPI_BYTES : EPI_BYTES + HALF_BYTES;
    const size_t smem = std::max<size_t>(tab.nst * stage_bytes, epi) + 1024;   // <= SMEM_MAX
    if (fwd) {
        dim3 grid(2 * groups(tab.gf), rows);
        dst_tc_kernel<0, EPI_H><<<grid, NTHREADS, smem, st>>>(
            g, tab, d->img, (const float*)a.src, (const float*)a.sub, a.sub_batches, spec, nullptr, nullptr, 0,
            nullptr);
    } else {
        // CTA pairs (clusters of 2): rank 0 the odd-k half, rank 1 the even-k half
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * groups(tab.gi), rows);
        cfg.blockDim = dim3(NTHREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        const float* add = (const float*)a.add;
        float* outp = (float*)a.out;
        const cudaError_t e = a.epi == EPI_H
            ? cudaLaunchKernelEx(&cfg, dst_tc_kernel<1, EPI_H>, g, tab, (const float*)d->img, (const float*)nullptr,
                                 (const float*)nullptr, 0, spec, outp, add, a.add_batches,
                                 (const int8_t*)p->d_mask)
            : cudaLaunchKernelEx(&cfg, dst_tc_kernel<1, EPI_ADJQ>, g, tab, (const float*)d->img,
                                 (const float*)nullptr, (const float*)nullptr, 0, spec, outp, add, a.add_batches,
                                 (const int8_t*)p->d_mask);
        if (e != cudaSuccess) return VD_ERR_CUDA;
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}

}  // namespace vd

extern "C" vd_status vd_device_error(int* flags, int reset)
{
    if (!flags) return VD_ERR_ARG;
    VD_CUDA_TRY(cudaMemcpyFromSymbol(flags, vd::g_tc_error, sizeof(int)));
    if (reset) {
        const int zero = 0;
        VD_CUDA_TRY(cudaMemcpyToSymbol(vd::g_tc_error, &zero, sizeof(int)));
    }
    return (vd_status)vd::qg_tile_error(flags, reset);
}
