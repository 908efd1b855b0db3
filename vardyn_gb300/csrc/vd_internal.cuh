// Internal declarations shared by the translation units of libvardyn_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include <mutex>
#include "../../include/vardyn_gb300.h"

#define VD_CUDA_TRY(expr)                                  \
    do {                                                   \
        cudaError_t _e = (expr);                           \
        if (_e != cudaSuccess) return VD_ERR_CUDA;         \
    } while (0)

namespace vd {
void count_launch();
}

// Every kernel launch site of the library is followed by this check; it also
// counts the launch (vd_launch_count).
#define VD_LAUNCH_CHECK()                  \
    do {                                   \
        vd::count_launch();                \
        VD_CUDA_TRY(cudaGetLastError());   \
    } while (0)

namespace vd {

// ---------------------------------------------------------------------------
// Grid constants passed to every QG kernel by value.
// ---------------------------------------------------------------------------
struct QGGeom {
    int ny, nx;
    long long fs;            // field stride = ny*nx
    double gf;               // g/f
    double gfc2;             // g*f/c^2
    double cu;               // -g/f/(4 dy)   (u = cu * 4-point y-difference)
    double cv;               //  g/f/(4 dx)
    double cx, cy;           // 1/(6 dx), 1/(6 dy)
    double idx2, idy2;       // 1/dx^2, 1/dy^2
    double Kx, Ky;           // Kdiffus/dx^2, Kdiffus/dy^2 (0 when absent)
    int hasK;
    const int8_t* mask;      // [ny][nx]
    const void* beta;        // T[ny][nx] or nullptr
    const void* fB;          // T[ny][nx] or nullptr
};

// DST-I / tridiagonal tables of one grid (typed by the plan dtype).
struct DSTTables {
    int n;        // interior columns = nx-2 (transform length)
    int my;       // interior rows = ny-2 (tridiagonal length)
    int ne, no;   // odd-output / even-output counts (ne = ceil(n/2), no = floor(n/2))
    int ncol_tiles;  // ceil(ne / DST_NC)
    int kpad;     // rows of the half matrices, padded to DST_KC
    int ldw;      // padded columns of the half matrices = ncol_tiles*DST_NC
    int lds;      // leading dimension of the spectral buffer
    void* Wodd;   // [kpad][ldw]  Wodd[p][t] = c sin(pi (p+1)(2t+1)/(n+1))
    void* WoddT;  // [kpad][ldw]  transpose of Wodd
    void* Weven;  // [kpad][ldw]  Weven[p][t] = c sin(pi (p+1)(2t+2)/(n+1)) (symmetric)
    void* trim;   // [my][lds] Thomas multipliers m_j per spectral column
    double tri_a; // off-diagonal g/f/dy^2
    void* tc;     // tensor-core images and tile table (float32 plans), or nullptr
    // float64 plans whose odd extension 2(n+1) factors into 2, 3, 5: the
    // FFT form of the transform (twiddles e^{-2 pi i m / L}, radix per stage)
    void* fft_tw = nullptr;
    int fft_L = 0, fft_nst = 0;
    int fft_rad[24] = {};
};

constexpr int DST_NC = 128;   // output columns per CTA tile
constexpr int DST_KC = 16;    // k rows per shared-memory chunk of the half matrices

// Epilogue kinds of the inverse transform
enum InvEpilogue { EPI_H = 0, EPI_ADJQ = 1 };

struct SolveArgs {
    // forward (physical -> spectral): x = src - sub over the interior
    const void* src;
    const void* sub;     // nullable; used for batches < sub_batches
    int sub_batches;
    // inverse (spectral -> physical)
    void* out;
    const void* add;     // EPI_H: hb (used for batches < add_batches); EPI_ADJQ: addend field
    int add_batches;
    int epi;
};

}  // namespace vd

struct vd_qg1l_plan {
    vd_qg1l_desc d;
    int nstage;
    double A[4][4];      // Butcher matrix with dt folded in
    double b[4];
    vd::QGGeom geom;     // device pointers inside
    vd::DSTTables dst;
    int8_t* d_mask;
    void* d_beta;
    void* d_fB;
    int device;
    vd_qg1l_schedule sched{};   // launch schedule of the inversion (0 = rule)
};

namespace vd {

size_t elem_size(int dtype);

// Helmholtz solve over `nf` fields (each [ny][nx]), spectral scratch `spec`.
template <typename T>
int helmholtz_solve(const vd_qg1l_plan* p, int nf, const SolveArgs& a, T* spec,
                    cudaStream_t st);

size_t spec_bytes(const vd_qg1l_plan* p, int nf);
int build_dst_tables(vd_qg1l_plan* p);
void free_dst_tables(vd_qg1l_plan* p);
int build_tc_images(vd_qg1l_plan* p);
void free_tc_images(vd_qg1l_plan* p);
// Whether a batch of nf fields fits the tensor-core pass (32-bit row offsets).
bool tc_fits(const vd_qg1l_plan* p, int nf);
// Whether the tensor-core pass runs for nf fields under the plan's schedule.
inline bool use_tc(const vd_qg1l_plan* p, int nf) { return p->dst.tc && tc_fits(p, nf) && p->sched.engine != 1; }
int dst_pass_tc(const vd_qg1l_plan* p, int nf, const SolveArgs& a, float* spec, bool fwd, cudaStream_t st);
// Neumann spectral Helmholtz solve of nf [nx][ny] fields (dst may equal src).
template <typename T>
int neumann_solve(const vd_neumann_plan* p, int nf, const T* src, T* dst, cudaStream_t st);
// ORs the stencil-tile error bits (8: a tile's bulk copies did not arrive)
// into *flags; reset != 0 clears them.
int qg_tile_error(int* flags, int reset);

// Kernel attributes (cudaFuncSetAttribute) apply to the device that is
// current when they are set. PerDeviceOnce runs a configuration function once
// for each device ordinal, on that device, and keeps its result, so plans on
// several GPUs of one process each launch with their attributes in place.
struct PerDeviceOnce {
    static constexpr int kMaxDevices = 64;
    std::mutex mu;
    bool done[kMaxDevices] = {};
    cudaError_t err[kMaxDevices] = {};
    template <typename F>
    cudaError_t run(F&& fn) {
        int dev = -1;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(mu);
        if (!done[dev]) {
            err[dev] = fn();
            done[dev] = true;
        }
        return err[dev];
    }
};

// Bump allocator over a caller workspace.
struct Arena {
    char* base;
    size_t cap;
    size_t off;
    void* take(size_t bytes) {
        size_t a = (off + 255) & ~size_t(255);
        if (a + bytes > cap) return nullptr;
        off = a + bytes;
        return base + a;
    }
};

}  // namespace vd
