// Galerkin assembly of the single-layer (V), double-layer (K) and hypersingular
// (W) operators and their first/second wavenumber derivatives on the GPU.
//
// Work decomposition (square P1 spaces, panel pairs i >= j as in
// galerkin_builder.cpp:958-1013):
//   * general pairs   -- one thread per (pair, job), p x p tensor Gauss points;
//   * singular pairs  -- one CTA per (coincident | adjacent pair, job), the
//                        n_c x n_c Duffy-mapped composite points (x2 for adjacent)
//                        split over the CTA and reduced in shared memory;
//   * gather          -- one thread per output entry: sums the four panel-pair
//                        contributions of a P1 dof pair and forms T(k) blocks.
// A "job" is one (wavenumber, refraction index) pair, so the two media of a
// T(k) and many wavenumbers are assembled by the same launch.
#pragma once
#include <cstdint>

#include "hbem_device.cuh"

namespace hbem {

// per-pair geometry flags (k independent), bit layout
enum : uint8_t {
    PF_DL0_ZERO = 1,     // double layer, triangle/set 0: v x n == 0 everywhere
    PF_DLT0_ZERO = 2,    // transposed double layer, set 0
    PF_DL1_ZERO = 4,     // double layer, set 1 (singular pairs)
    PF_DLT1_ZERO = 8,    // transposed double layer, set 1
    PF_TDT0_ZERO = 16,   // tangent . tangent == 0, set 0
    PF_TDT1_ZERO = 32,   // set 1
};

enum PairKind : int { PK_COINC = 0, PK_ADJ = 1, PK_GEN = 2 };

struct SingularTask {
    int i, j, kind, swap;
};

// device view of a mesh + quadrature
struct DevMesh {
    int n;            // panels
    int p;            // Gauss order
    int nc;           // composite nodes
    int lines;        // all panels are straight lines
    const int* kind;          // [n]
    const double* par;        // [n][5]  line: x1 y1 x2 y2 ; arc: cx cy r phi0 phi1
    const double* xg;         // [p]
    const double* wg;         // [p]
    const double* xc;         // [nc]
    const double* wc;         // [nc]
    const cplx* gpt;          // [n][p] points at the general nodes
    const cplx* gtan;         // [n][p] tangents
    const double* gtn;        // [n][p] tangent norms
    const cplx* ends;         // [n][2] start/end (the [-1,1] map at -1/+1)
    const uint8_t* flags;     // [n(n+1)/2] per lower-triangle pair
    const int* gorder = nullptr;   // [n(n-1)/2] strictly-lower pairs by distance (thread-per-pair order), or null
    const double* sgeo = nullptr;   // [ntasks][2][kSGeoFields][nc*nc] singular-pair point data, or null
};

// k-independent data of one composite quadrature point of a singular pair:
//   coincident (set 0 serves both triangles): |v|^2, |v|, 2 tau_i.tau_j, dl0, dl1, w, s, t,
//   adjacent (set K):                         |v|^2, |v|, 2 tau_i.tau_j, dl, dlt, w, x, y,
// then 1/|v| and log|v| for both (0 where |v| = 0)
constexpr int kSGeoFields = 10;

// one (k, c) job
struct Job {
    double kre, kim, c;
};

// a mesh of a many-mesh launch: its device view and singular-pair list
struct MultiMesh {
    DevMesh M;
    const SingularTask* tasks;
    int ntasks;
};

// a job of a many-mesh launch: (k, c), the mesh, and the offset (complex entries)
// of the job's pair-block array in the launch's scratch
struct MultiJob {
    Job job;
    int mesh;
    long long loc;
};

// number of complex entries of a pair's local block set per derivative order:
// DL(2x2) DLt(2x2) HY(2x2) SL(2x2)
constexpr int kLocPerD = 16;

__host__ __device__ __forceinline__ long long tri_index(long long i, long long j) { return i * (i + 1) / 2 + j; }

}  // namespace hbem
