// Batched form: hundreds of independent meshes assembled in one persistent
// launch and solved by one batched Jacobi-PCG replayed from a CUDA graph.
//
// The batch is viewed as one block-diagonal system.  Mesh b owns global rows
// [dof_off[b], dof_off[b+1]) and the triplet range [trip_off[b], trip_off[b+1])
// of the batch COO, filled in the order of AssembleMatrixLocally on mesh b
// alone (assemble/assembler.h:114-186) with row/col shifted by dof_off[b].
// The existing fix (lfg_fix_*) and COO->CSR (lfg_csr_from_coo) then act on
// the whole batch at once; only assembly and the solve need batch awareness.
//
// Assembly: work items are tiles of T consecutive cells of one mesh (T =
// threads per CTA); a persistent grid loops over the items, finds the item's
// mesh by binary search in the tile prefix, and runs the df32 triangle body
// for the mesh's degree (lfg_elem.h).  T and the CTAs per SM are chosen by
// timing the candidates on the first call (the autotuner).
//
// Solve: rows are cut into chunks that never straddle two meshes; every PCG
// kernel works chunk by chunk and every per-mesh scalar (step length,
// direction update, residual) is a sum of that mesh's chunk partials in a
// fixed order, so each block of the system follows exactly its own PCG.
// Converged meshes are frozen (no more updates) while the others continue.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lfg_api.h"
#include "lfg_elem.h"
#include "lfg_internal.h"

namespace lfg {

struct BatchMesh {
  const double2* xy;
  const int4* cells;
  const int32_t* cell_dofs;
  const int64_t* tri_offset;
  int n_cell;
  int degree;
  int64_t ncells;
  int64_t dof_off;
  int64_t cell_off;
  int64_t trip_off;
};

}  // namespace lfg

struct lfg_batch {
  lfg::CtxRef ref;
  lfg_ctx* ctx = nullptr;
  int nb = 0;
  std::vector<lfg_space*> spaces;
  std::vector<int64_t> dof_off, cell_off, trip_off;
  lfg::DevBuf meshes;  // BatchMesh[nb]
  int max_degree = 0;
  // autotuning result
  bool tuned = false;
  int threads = 128, ctas_per_sm = 0;
  double best_ms = 0.0;
  // PCG chunks (chunk_rows rows each, never straddling two meshes)
  lfg::DevBuf chunk_mesh, chunk_start, mesh_chunk_off;
  int64_t nchunks = 0;
  int chunk_rows = 0;
  std::vector<int64_t> h_mesh_chunk_off;
  // rows per chunk of the batched PCG per precision (0 FP64, 1 mixed), chosen
  // by timing the candidates on the first solve in that precision
  bool solve_tuned[2] = {false, false};
  int solve_chunk_rows[2] = {2048, 2048};
  double solve_rate[2] = {0.0, 0.0};  // row-iterations per second of the chosen shape
  // grouped solver: meshes packed into groups of at most this many bytes of
  // solver data (0: every mesh in one lock-step sweep)
  double solve_group_bytes = 0.0;
};

namespace lfg {
void EnsureIncidence(lfg_space* sp);
namespace {

using elem::f2;

constexpr int kMaxBatchThreads = 256;

struct BatchArgs {
  const BatchMesh* meshes;
  int nb;
  const int64_t* tile_prefix;  // nb + 1
  int64_t total_tiles;
  lfg_triplet* out;
  const double* alpha;  // per batch cell, or null (constant alpha_value)
  double alpha_value;
  const double* gamma;
  double gamma_value;
  const f2* tabs[4];    // df32 R tables per degree (index = degree)
  const double* tabs64[4];  // FP64 R tables per degree
  unsigned long long* fallback;
};

__device__ __forceinline__ void StoreTripletB(lfg_triplet* p, int r, int c, double v) {
  const long long bits = __double_as_longlong(v);
  *reinterpret_cast<int4*>(p) = make_int4(r, c, static_cast<int>(bits & 0xffffffffll), static_cast<int>(bits >> 32));
}

template <int N>
__device__ __forceinline__ int UpperIdx(int i, int j) {
  const int a = i < j ? i : j, b = i < j ? j : i;
  return a * N - (a * (a - 1)) / 2 + (b - a);
}

template <int DEG, bool MASS>
__device__ void BatchTile(const BatchArgs& A, const BatchMesh& m, int64_t first, int ncell, unsigned char* smem) {
  constexpr int N = (DEG + 1) * (DEG + 2) / 2;
  constexpr int E = N * (N + 1) / 2;
  constexpr int NN = N * N;
  const int T = blockDim.x;
  double* svals = reinterpret_cast<double*>(smem);
  int64_t* soff = reinterpret_cast<int64_t*>(svals + T * E);
  int* sdofs = reinterpret_cast<int*>(soff + T);
  if (threadIdx.x < ncell) {
    const int64_t c = first + threadIdx.x;
    const int4 cn = m.cells[c];
    const double2 v0 = m.xy[cn.x], v1 = m.xy[cn.y], v2 = m.xy[cn.z];
    const double jac[4] = {v1.x - v0.x, v2.x - v0.x, v1.y - v0.y, v2.y - v0.y};
    const double al = A.alpha ? A.alpha[m.cell_off + c] : A.alpha_value;
    const double ga = MASS ? (A.gamma ? A.gamma[m.cell_off + c] : A.gamma_value) : 0.0;
    double* vals = svals + threadIdx.x * E;
    if (elem::DfSafe(jac[0]) && elem::DfSafe(jac[1]) && elem::DfSafe(jac[2]) && elem::DfSafe(jac[3]) &&
        elem::DfSafe(al) && elem::DfSafe(ga)) {
      elem::TriaUniformDF<E, MASS>(jac, al, ga, A.tabs[DEG], vals);
    } else {
      elem::TriaUniformF64<E, MASS>(jac, al, ga, A.tabs64[DEG], vals);
      atomicAdd(A.fallback, 1ull);
    }
#pragma unroll
    for (int i = 0; i < N; ++i)
      sdofs[threadIdx.x * N + i] = m.cell_dofs[c * m.n_cell + i] + static_cast<int>(m.dof_off);
    soff[threadIdx.x] = m.trip_off + m.tri_offset[c];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < ncell * NN; q += T) {
    const int cl = q / NN, w = q - cl * NN;
    const int i = w / N, j = w - i * N;
    StoreTripletB(A.out + soff[cl] + w, sdofs[cl * N + i], sdofs[cl * N + j], svals[cl * E + UpperIdx<N>(i, j)]);
  }
  __syncthreads();
}

template <bool MASS>
__global__ void __launch_bounds__(kMaxBatchThreads) BatchAssembleKernel(BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_mesh;
  for (int64_t t = blockIdx.x; t < A.total_tiles; t += gridDim.x) {
    if (threadIdx.x == 0) {  // mesh of this tile: last b with tile_prefix[b] <= t
      int lo = 0, hi = A.nb - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.tile_prefix[mid] <= t) lo = mid;
        else hi = mid - 1;
      }
      s_mesh = lo;
    }
    __syncthreads();
    const BatchMesh m = A.meshes[s_mesh];
    const int64_t first = (t - A.tile_prefix[s_mesh]) * blockDim.x;
    const int64_t left = m.ncells - first;
    const int ncell = static_cast<int>(left < blockDim.x ? left : blockDim.x);
    __syncthreads();
    switch (m.degree) {
      case 1: BatchTile<1, MASS>(A, m, first, ncell, smem); break;
      case 2: BatchTile<2, MASS>(A, m, first, ncell, smem); break;
      case 3: BatchTile<3, MASS>(A, m, first, ncell, smem); break;
    }
  }
}

size_t StagePerCell(int degree) {
  const int N = (degree + 1) * (degree + 2) / 2, E = N * (N + 1) / 2;
  return E * 8 + 8 + N * 4;
}

// ------------------------------------------------------------ batched PCG
constexpr int kChunk = 2048;  // rows per chunk until the solver autotuner has chosen
constexpr int kPB = 256;  // threads per block of the PCG kernels
constexpr int kLanes = 8;

struct Chunks {
  const int32_t* mesh;        // chunk -> mesh
  const int64_t* start;       // chunk -> first row (nchunks + 1: start[nchunks] = total rows)
  const int64_t* mesh_chunk;  // mesh -> first chunk (nb + 1)
  int64_t nchunks;
};

__device__ double BlockReduce(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

// Per-mesh PCG scalars on the device (rz[cur] = <r, z> of the current
// residual; the update kernel writes rz[cur ^ 1]).
struct MeshScal {
  double rz[2];
  double alpha, beta, rr, pq;
  unsigned int cnt;  // chunks of this mesh finished in the current kernel
  unsigned int pad;
};

// Called by every block after it wrote the partial(s) of chunk c of mesh b:
// true for the block that finished the mesh's last chunk (counter after a
// fence; no block waits for another).  That block then reduces the mesh's
// chunk partials in chunk order.
__device__ __forceinline__ bool MeshDone(MeshScal* ms, int b, unsigned int nch) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ms[b].cnt, 1u) == nch - 1;
  }
  __syncthreads();
  return last;
}

__device__ double MeshPartSum(const double* part, int stride, int off, int64_t c0, int64_t c1, double* red) {
  double v = 0.0;
  for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) v += __ldcg(part + c * stride + off);
  v = BlockReduce(v, red);
  return v;  // valid in thread 0
}

template <class T>
struct BDot {
  double v = 0.0;
  __device__ void add(T a, T b) { v = fma(a, b, v); }
  __device__ double get() const { return v; }
};
template <>
struct BDot<float> {
  float v = 0.0f;
  __device__ void add(float a, float b) { v = fmaf(a, b, v); }
  __device__ double get() const { return static_cast<double>(v); }
};

struct Sell {
  const int64_t* ptr;
  const int32_t* col;
};

// q = A p on the chunk's rows (SELL-32; thread per row), <p, q> per mesh
// -> alpha_b.
// With `rowsum` (the FP32 copy) each row is applied in difference form,
// sum_k a_rk (p_k - p_r) + s_r p_r with the FP64 row sum s_r rounded once,
// which keeps the FP32 operator close to A on its smooth modes.
template <class T>
__global__ void __launch_bounds__(kPB) BSpmvKernel(Chunks C, Sell M, const T* __restrict__ val,
                                                   const T* __restrict__ rowsum,
                                                   const T* __restrict__ p, T* __restrict__ q,
                                                   const int32_t* __restrict__ frozen, int cur,
                                                   double* __restrict__ part, MeshScal* __restrict__ ms) {
  __shared__ double red[32];
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const int b = C.mesh[c];
    if (frozen[b]) continue;  // uniform per block
    BDot<T> acc;
    for (int64_t r = C.start[c] + threadIdx.x; r < C.start[c + 1]; r += blockDim.x) {
      const int64_t sl = r >> 5, lane = r & 31;
      const int64_t b0 = M.ptr[sl];
      const int w = static_cast<int>((M.ptr[sl + 1] - b0) >> 5);
      const int32_t* cp = M.col + b0 + lane;
      const T* vp = val + b0 + lane;
      T sum = T(0);
      if (rowsum) {
        const T pr = p[r];
#pragma unroll 4
        for (int k = 0; k < w; ++k) sum = fma(vp[k * 32], p[cp[k * 32]] - pr, sum);
        sum = fma(rowsum[r], pr, sum);
      } else {
#pragma unroll 4
        for (int k = 0; k < w; ++k) sum = fma(vp[k * 32], p[cp[k * 32]], sum);
      }
      q[r] = sum;
      acc.add(p[r], sum);
    }
    const double tot = BlockReduce(acc.get(), red);
    if (threadIdx.x == 0) part[c] = tot;
    const int64_t c0 = C.mesh_chunk[b], c1 = C.mesh_chunk[b + 1];
    if (MeshDone(ms, b, static_cast<unsigned int>(c1 - c0))) {
      const double pq = MeshPartSum(part, 1, 0, c0, c1, red);
      if (threadIdx.x == 0) {
        ms[b].pq = pq;
        ms[b].alpha = pq != 0.0 ? ms[b].rz[cur] / pq : 0.0;
        ms[b].cnt = 0;
      }
    }
    __syncthreads();
  }
}

// x += alpha_b p; r -= alpha_b q; z = D^-1 r; <r, z>, <r, r> per mesh ->
// rz[cur ^ 1], rr, beta_b.
template <class T>
__global__ void __launch_bounds__(kPB) BUpdateKernel(Chunks C, const T* __restrict__ dinv, const T* __restrict__ p,
                                                     const T* __restrict__ q, T* __restrict__ x, T* __restrict__ r,
                                                     T* __restrict__ z, const int32_t* __restrict__ frozen, int cur,
                                                     double* __restrict__ part, MeshScal* __restrict__ ms) {
  __shared__ double red[32];
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const int b = C.mesh[c];
    if (frozen[b]) continue;
    const T alpha = static_cast<T>(ms[b].alpha);
    BDot<T> arz, arr;
    // U elements per thread and trip, loads first (more loads in flight)
    constexpr int U = sizeof(T) == 8 ? 2 : 4;
    const int64_t e = C.start[c + 1];
    for (int64_t i0 = C.start[c] + threadIdx.x; i0 < e; i0 += U * blockDim.x) {
      T pv[U], qv[U], xv[U], rv[U], dv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = i0 + u * blockDim.x;
        if (i < e) {
          pv[u] = p[i]; qv[u] = q[i]; xv[u] = x[i]; rv[u] = r[i]; dv[u] = dinv[i];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = i0 + u * blockDim.x;
        if (i < e) {
          x[i] = fma(alpha, pv[u], xv[u]);
          const T ri = fma(-alpha, qv[u], rv[u]);
          r[i] = ri;
          const T zi = dv[u] * ri;
          z[i] = zi;
          arz.add(ri, zi);
          arr.add(ri, ri);
        }
      }
    }
    const double s1 = BlockReduce(arz.get(), red);
    const double s2 = BlockReduce(arr.get(), red);
    if (threadIdx.x == 0) {
      part[2 * c] = s1;
      part[2 * c + 1] = s2;
    }
    const int64_t c0 = C.mesh_chunk[b], c1 = C.mesh_chunk[b + 1];
    if (MeshDone(ms, b, static_cast<unsigned int>(c1 - c0))) {
      const double rz = MeshPartSum(part, 2, 0, c0, c1, red);
      const double rr = MeshPartSum(part, 2, 1, c0, c1, red);
      if (threadIdx.x == 0) {
        const double rz_old = ms[b].rz[cur];
        ms[b].rz[cur ^ 1] = rz;
        ms[b].beta = rz_old != 0.0 ? rz / rz_old : 0.0;
        ms[b].rr = rr;
        ms[b].cnt = 0;
      }
    }
    __syncthreads();
  }
}

// p = z + beta_b p.
template <class T>
__global__ void __launch_bounds__(kPB) BDirectionKernel(Chunks C, const T* __restrict__ z, T* __restrict__ p,
                                                        const int32_t* __restrict__ frozen,
                                                        const MeshScal* __restrict__ ms) {
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const int b = C.mesh[c];
    if (frozen[b]) continue;
    const T beta = static_cast<T>(ms[b].beta);
    constexpr int U = sizeof(T) == 8 ? 2 : 4;
    const int64_t e = C.start[c + 1];
    for (int64_t i0 = C.start[c] + threadIdx.x; i0 < e; i0 += U * blockDim.x) {
      T pv[U], zv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = i0 + u * blockDim.x;
        if (i < e) {
          pv[u] = p[i];
          zv[u] = z[i];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = i0 + u * blockDim.x;
        if (i < e) p[i] = fma(beta, pv[u], zv[u]);
      }
    }
  }
}

// z = D^-1 r, p = z; rz[0], rr per mesh; beta = 0 (so the first direction
// update keeps p = z).
template <class T>
__global__ void __launch_bounds__(kPB) BStartKernel(Chunks C, const T* __restrict__ dinv, const T* __restrict__ r,
                                                    T* __restrict__ z, T* __restrict__ p,
                                                    const int32_t* __restrict__ frozen, double* __restrict__ part,
                                                    MeshScal* __restrict__ ms) {
  __shared__ double red[32];
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const int b = C.mesh[c];
    if (frozen[b]) continue;
    double arz = 0.0, arr = 0.0;
    for (int64_t i = C.start[c] + threadIdx.x; i < C.start[c + 1]; i += blockDim.x) {
      const T ri = r[i];
      const T zi = dinv[i] * ri;
      z[i] = zi;
      p[i] = zi;
      arz = fma(static_cast<double>(ri), static_cast<double>(zi), arz);
      arr = fma(static_cast<double>(ri), static_cast<double>(ri), arr);
    }
    const double s1 = BlockReduce(arz, red);
    const double s2 = BlockReduce(arr, red);
    if (threadIdx.x == 0) {
      part[2 * c] = s1;
      part[2 * c + 1] = s2;
    }
    const int64_t c0 = C.mesh_chunk[b], c1 = C.mesh_chunk[b + 1];
    if (MeshDone(ms, b, static_cast<unsigned int>(c1 - c0))) {
      const double rz = MeshPartSum(part, 2, 0, c0, c1, red);
      const double rr = MeshPartSum(part, 2, 1, c0, c1, red);
      if (threadIdx.x == 0) {
        ms[b].rz[0] = rz;
        ms[b].rz[1] = 0.0;
        ms[b].alpha = 0.0;
        ms[b].beta = 0.0;
        ms[b].rr = rr;
        ms[b].cnt = 0;
      }
    }
    __syncthreads();
  }
}

// Row r of a CSR matrix times x by the 8 lanes of a group (fixed shuffle order).
template <class T>
__device__ __forceinline__ T RowDotB(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                     const T* __restrict__ val, const T* __restrict__ x, int64_t r, int64_t end,
                                     int sub) {
  T s = T(0);
  if (r < end)
    for (int q = rp[r] + sub; q < rp[r + 1]; q += kLanes) s = fma(val[q], x[col[q]], s);
#pragma unroll
  for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kLanes);
  return s;
}

// r = b - A x (FP64) and rr partials; optional x == null means x = 0.  With
// `only`, meshes b with only[b] == 0 are skipped (their rows and partials
// keep their values).
__global__ void __launch_bounds__(kPB) BResidualKernel(Chunks C, const int32_t* __restrict__ rp,
                                                       const int32_t* __restrict__ col, const double* __restrict__ val,
                                                       const double* __restrict__ x, const double* __restrict__ b,
                                                       double* __restrict__ r, double* __restrict__ rr,
                                                       const int32_t* __restrict__ only = nullptr) {
  __shared__ double red[32];
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    if (only && !only[C.mesh[c]]) continue;  // uniform per block
    const int64_t s = C.start[c], e = C.start[c + 1];
    const int sub = threadIdx.x % kLanes, grp = threadIdx.x / kLanes;
    double acc = 0.0;
    for (int64_t wb = s; wb < e; wb += kPB / kLanes) {
      const int64_t i = wb + grp;
      const double v = x ? RowDotB<double>(rp, col, val, x, i, e, sub) : 0.0;
      if (sub == 0 && i < e) {
        const double ri = b[i] - v;
        r[i] = ri;
        acc = fma(ri, ri, acc);
      }
    }
    const double tot = BlockReduce(acc, red);
    if (threadIdx.x == 0) rr[c] = tot;
  }
}

// r32 = r64 * scale[mesh], d32 = 0 (mixed-precision inner start)
__global__ void BScaleKernel(Chunks C, const double* __restrict__ r, const double* __restrict__ scale,
                             float* __restrict__ r32, float* __restrict__ d32) {
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const double s = scale[C.mesh[c]];
    for (int64_t i = C.start[c] + threadIdx.x; i < C.start[c + 1]; i += blockDim.x) {
      r32[i] = static_cast<float>(r[i] * s);
      d32[i] = 0.0f;
    }
  }
}

// x += sign * d32 / scale[mesh] for the meshes with sel[mesh] set (the FP32
// correction at a residual replacement; sign -1 takes it back).
__global__ void BApplyKernel(Chunks C, const float* __restrict__ d, const double* __restrict__ scale,
                             const int32_t* __restrict__ sel, double sign, double* __restrict__ x) {
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const int b = C.mesh[c];
    if (!sel[b]) continue;
    const double f = sign / scale[b];
    for (int64_t i = C.start[c] + threadIdx.x; i < C.start[c + 1]; i += blockDim.x)
      x[i] = fma(static_cast<double>(d[i]), f, x[i]);
  }
}

// Residual replacement for the meshes with sel[mesh] set: r32 = r64 *
// scale[mesh] (the FP64 true residual), z = D^-1 r32, d32 = 0; rz[0], rr and
// beta = rz[0] / rz[1] per mesh from the new residual (p is kept).
__global__ void __launch_bounds__(kPB) BReplaceKernel(Chunks C, const double* __restrict__ r64,
                                                      const double* __restrict__ scale,
                                                      const float* __restrict__ dinv, float* __restrict__ r,
                                                      float* __restrict__ z, float* __restrict__ d,
                                                      const int32_t* __restrict__ sel, double* __restrict__ part,
                                                      MeshScal* __restrict__ ms) {
  __shared__ double red[32];
  for (int64_t c = blockIdx.x; c < C.nchunks; c += gridDim.x) {
    const int b = C.mesh[c];
    if (!sel[b]) continue;
    const double sc = scale[b];
    double arz = 0.0, arr = 0.0;
    for (int64_t i = C.start[c] + threadIdx.x; i < C.start[c + 1]; i += blockDim.x) {
      const float ri = static_cast<float>(r64[i] * sc);
      const float zi = dinv[i] * ri;
      r[i] = ri;
      z[i] = zi;
      d[i] = 0.0f;
      arz = fma(static_cast<double>(ri), static_cast<double>(zi), arz);
      arr = fma(static_cast<double>(ri), static_cast<double>(ri), arr);
    }
    const double s1 = BlockReduce(arz, red);
    const double s2 = BlockReduce(arr, red);
    if (threadIdx.x == 0) {
      part[2 * c] = s1;
      part[2 * c + 1] = s2;
    }
    const int64_t c0 = C.mesh_chunk[b], c1 = C.mesh_chunk[b + 1];
    if (MeshDone(ms, b, static_cast<unsigned int>(c1 - c0))) {
      const double rz = MeshPartSum(part, 2, 0, c0, c1, red);
      const double rr = MeshPartSum(part, 2, 1, c0, c1, red);
      if (threadIdx.x == 0) {
        // the search direction is kept (beta from the new and the last
        // recursive <r, z>) unless the replaced residual exceeds the
        // recursive one by more than 16: the FP32 recursion had run past what
        // it can resolve, its direction no longer belongs to this residual,
        // and the block restarts from p = z
        const double rz_old = ms[b].rz[1];
        ms[b].beta = rz_old > 0.0 && rz <= 16.0 * rz_old ? rz / rz_old : 0.0;
        ms[b].rz[0] = rz;
        ms[b].rr = rr;
        ms[b].cnt = 0;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------ grouped PCG
// The lock-step solver streams every mesh's matrix and vectors from HBM on
// every iteration.  The grouped solver instead packs meshes into groups whose
// solver data fits in L2 and iterates one group at a time in one cooperative,
// persistent launch per `check_every` iterations, so a group's matrix and
// vectors stay in L2 across iterations.  The iteration is the Chronopoulos-
// Gear form of Jacobi-PCG (one reduction per iteration):
//   phase A  p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s,
//            u = D^-1 r                                   (row-local)
//   barrier
//   phase B  w = A u; <r, u>, <w, u>, <r, r> per mesh      (gathers u)
//   barrier
//   scalars  beta = g / g_prev, alpha = g / (d - beta g / alpha_prev)
// (s = A p throughout; at a mesh's (re)start beta = 0 and alpha = g / d, and
// a non-positive denominator restarts the same way).  The group's rows are
// cut into lanesets of at most 32 consecutive rows of one mesh; block k owns
// a contiguous range of at most kGMaxLs lanesets, one warp per laneset, so a
// block reads and writes its own rows in every phase and only the gathers of
// u and the partial sums cross blocks (read through L2).  Consecutive
// lanesets of one mesh within a block form a run; a run's three sums are
// written once per iteration, and every block that needs a mesh's scalars
// sums the mesh's run partials itself, in run order with the same warp tree,
// so all blocks get the same bits and the result does not depend on timing.
// Within a phase no location is both written and read by different threads,
// and the barrier's acquire orders each phase after the previous one, so the
// vectors are read with ordinary (L1-cached) loads.  The per-mesh scalars
// (a mesh's owner sets its frozen flag while other blocks may read it) and
// the partial sums are read through L2.
constexpr int kGThreads = 512;
constexpr int kGMinBlocks = 2;  // resident blocks per SM the kernel is compiled for
constexpr int kGWarps = kGThreads / 32;
constexpr int kGMaxLs = 64;                     // lanesets (so also runs) per block
constexpr unsigned int kGBarPolls = 1u << 22;   // bounded barrier polls (about a second)

struct GridBar {
  unsigned int arrive;  // monotone arrival count of the launch (zeroed before it)
  int err;              // a barrier gave up
};

// Per-mesh scalars of the grouped solver, published by the block that owns
// the mesh's first run (read by the other blocks and by the host).
struct GMeshScal {
  double gam[2];   // <r, u> of iteration i in slot i & 1
  double alp[2];   // alpha of iteration i in slot i & 1
  double rr;       // <r, r> at the last stopping test
  int32_t frozen;  // converged (or not part of the run)
  int32_t it;      // iteration index of the last stopping test
  int32_t fresh;   // iteration at which the mesh (re)starts (beta = 0 there)
  int32_t pad;
};

struct GGroup {
  const int64_t* ls_row;    // laneset -> first row
  const int32_t* ls_n;      // laneset -> rows (1..32)
  const int32_t* ls_run;    // laneset -> run
  const int32_t* run_mesh;  // run -> mesh
  const int32_t* run_ls;    // run -> first laneset (nrun + 1)
  const int32_t* run_m0;    // run -> first run of its mesh
  const int32_t* run_m1;    // run -> one past the last run of its mesh
  const int32_t* blk_ls;    // block -> first laneset (grid + 1)
  const int32_t* blk_run;   // block -> first run (grid + 1)
};

template <class T>
struct GArgs {
  GGroup g;
  Sell M;
  const T* val;
  const T* rowsum;     // difference form (FP32) or null
  const T* dinv;
  T *x, *r, *u, *w, *p, *s;
  const double* r64;   // (re)start from r = r64 * scale[mesh] with x = 0 (mixed), else from r
  const double* scale;
  const int32_t* sel;  // (re)start only the meshes with sel[mesh] (null: the whole group)
  double* part;        // per run: <r, u>, <w, u>, <r, r>
  GMeshScal* gs;
  const double* target;  // per mesh: stop when <r, r> <= target
  int iters;             // iterations of this launch
  int i0;                // index of its first iteration within the group's run
  int start;             // (re)start phase first
  GridBar* bar;
};

// Grid barrier of a cooperative launch: every block adds one to a monotone
// counter (release) and waits (acquire loads) until it reaches epoch x grid.
// A wait gives up after kGBarPolls polls or when another block gave up; the
// block then reports false and leaves the kernel.
__device__ __forceinline__ bool GBarSync(GridBar* g, unsigned int& epoch, int* s_ok) {
  __syncthreads();
  ++epoch;
  if (threadIdx.x == 0) {
    const unsigned int want = epoch * gridDim.x;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&g->arrive) : "memory");
    unsigned int v = 0, polls = 0;
    int ok = 1;
    while (true) {
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(&g->arrive) : "memory");
      if (static_cast<int>(v - want) >= 0) break;
      if (++polls > kGBarPolls || *reinterpret_cast<volatile int*>(&g->err)) {
        ok = 0;
        atomicExch(&g->err, 1);
        break;
      }
      __nanosleep(32);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

__device__ __forceinline__ double WarpSum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
__global__ void __launch_bounds__(kGThreads, kGMinBlocks) BGroupCgKernel(GArgs<T> a) {
  __shared__ double s_ls[kGMaxLs][3];           // laneset sums of phase B
  __shared__ double s_al[kGMaxLs], s_be[kGMaxLs];  // per run of this block
  __shared__ int s_act[kGMaxLs];
  __shared__ int s_ok;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const GGroup& G = a.g;
  const int ls0 = G.blk_ls[blockIdx.x], ls1 = G.blk_ls[blockIdx.x + 1];
  const int rn0 = G.blk_run[blockIdx.x], rn1 = G.blk_run[blockIdx.x + 1];
  unsigned int epoch = 0;
  const bool restart_all = a.start && !a.sel;

  // phase B on the lanesets whose run is live: w = A u, the three sums per
  // laneset, then per run (in laneset order) into part
  auto phase_b = [&](bool restart) {
    for (int l = ls0 + warp; l < ls1; l += kGWarps) {
      const int j = G.ls_run[l] - rn0;
      const bool live = restart ? (restart_all || a.sel[G.run_mesh[rn0 + j]]) : s_act[j] != 0;
      if (!live) continue;
      const int64_t row = G.ls_row[l] + lane;
      double g = 0.0, d = 0.0, rr = 0.0;
      if (lane < G.ls_n[l]) {
        const int64_t slc = row >> 5, li = row & 31;
        const int64_t b0 = a.M.ptr[slc];
        const int wd = static_cast<int>((a.M.ptr[slc + 1] - b0) >> 5);
        const int32_t* cp = a.M.col + b0 + li;
        const T* vp = a.val + b0 + li;
        const T ur = a.u[row];
        const T sh = a.rowsum ? ur : T(0);  // difference form: a_rk (u_k - u_r)
        T sum = T(0);
        // eight columns at a time: all their loads, then all their gathers
        // (positions past the slice width add a zero term)
        for (int k = 0; k < wd; k += 8) {
          int32_t c[8];
          T v[8], g[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const bool in = k + j < wd;
            c[j] = in ? __ldg(cp + (k + j) * 32) : static_cast<int32_t>(row);
            v[j] = in ? __ldg(vp + (k + j) * 32) : T(0);
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) g[j] = a.u[c[j]];
#pragma unroll
          for (int j = 0; j < 8; ++j) sum = fma(v[j], g[j] - sh, sum);
        }
        if (a.rowsum) sum = fma(a.rowsum[row], ur, sum);
        a.w[row] = sum;
        const double rv = static_cast<double>(a.r[row]);
        g = rv * static_cast<double>(ur);
        d = static_cast<double>(sum) * static_cast<double>(ur);
        rr = rv * rv;
      }
      g = WarpSum(g);
      d = WarpSum(d);
      rr = WarpSum(rr);
      if (lane == 0) {
        s_ls[l - ls0][0] = g;
        s_ls[l - ls0][1] = d;
        s_ls[l - ls0][2] = rr;
      }
    }
    __syncthreads();
    for (int j = warp; j < rn1 - rn0; j += kGWarps) {
      const int run = rn0 + j;
      const bool live = restart ? (restart_all || a.sel[G.run_mesh[run]]) : s_act[j] != 0;
      if (!live) continue;
      const int f0 = G.run_ls[run] - ls0, f1 = G.run_ls[run + 1] - ls0;
      double g = 0.0, d = 0.0, rr = 0.0;
      for (int q = f0 + lane; q < f1; q += 32) {
        g += s_ls[q][0];
        d += s_ls[q][1];
        rr += s_ls[q][2];
      }
      g = WarpSum(g);
      d = WarpSum(d);
      rr = WarpSum(rr);
      if (lane == 0) {
        a.part[3 * run] = g;
        a.part[3 * run + 1] = d;
        a.part[3 * run + 2] = rr;
      }
    }
  };

  if (a.start) {
    // (re)start: r (from r64 in the mixed form, with x = 0), u = D^-1 r, p = s = 0
    for (int l = ls0 + warp; l < ls1; l += kGWarps) {
      const int mesh = G.run_mesh[G.ls_run[l]];
      if (!restart_all && !a.sel[mesh]) continue;
      if (lane >= G.ls_n[l]) continue;
      const int64_t row = G.ls_row[l] + lane;
      T ri;
      if (a.r64) {
        ri = static_cast<T>(a.r64[row] * a.scale[mesh]);
        a.r[row] = ri;
        a.x[row] = T(0);
      } else {
        ri = a.r[row];
      }
      a.u[row] = a.dinv[row] * ri;
      a.p[row] = T(0);
      a.s[row] = T(0);
    }
    if (!GBarSync(a.bar, epoch, &s_ok)) return;
    phase_b(true);
    if (!GBarSync(a.bar, epoch, &s_ok)) return;
  }
  for (int k = 0;; ++k) {
    const int i = a.i0 + k;
    // ---- scalars of every run's mesh, the stopping test
    for (int j = warp; j < rn1 - rn0; j += kGWarps) {
      const int run = rn0 + j, b = G.run_mesh[run];
      const int m0 = G.run_m0[run], m1 = G.run_m1[run];
      // read once per warp: the flag may be set by the mesh's owner during
      // this very phase (its test gives every block the same answer)
      const int live = __shfl_sync(0xffffffffu, lane == 0 ? !*reinterpret_cast<volatile int32_t*>(&a.gs[b].frozen) : 0, 0);
      if (!live) {
        if (lane == 0) s_act[j] = 0;
        continue;
      }
      double g = 0.0, d = 0.0, rr = 0.0;
      for (int q = m0 + lane; q < m1; q += 32) {
        g += __ldcg(a.part + 3 * q);
        d += __ldcg(a.part + 3 * q + 1);
        rr += __ldcg(a.part + 3 * q + 2);
      }
      g = WarpSum(g);
      d = WarpSum(d);
      rr = WarpSum(rr);
      if (lane == 0) {
        const bool conv = !(rr > a.target[b]);
        double al = d > 0.0 ? g / d : 0.0, be = 0.0;
        if (__ldcg(&a.gs[b].fresh) != i) {
          const double g0 = __ldcg(&a.gs[b].gam[(i - 1) & 1]), a0 = __ldcg(&a.gs[b].alp[(i - 1) & 1]);
          const double bt = g0 != 0.0 ? g / g0 : 0.0;
          const double den = a0 != 0.0 ? d - bt * g / a0 : 0.0;
          if (den > 0.0 && den < INFINITY) {
            be = bt;
            al = g / den;
          }
        }
        s_al[j] = al;
        s_be[j] = be;
        s_act[j] = !conv && k < a.iters;
        if (run == m0) {
          a.gs[b].gam[i & 1] = g;
          a.gs[b].alp[i & 1] = al;
          a.gs[b].rr = rr;
          a.gs[b].it = i;
          if (conv) a.gs[b].frozen = 1;
        }
      }
    }
    __syncthreads();
    if (k == a.iters) break;
    // ---- phase A
    for (int l = ls0 + warp; l < ls1; l += kGWarps) {
      const int j = G.ls_run[l] - rn0;
      if (!s_act[j] || lane >= G.ls_n[l]) continue;
      const int64_t row = G.ls_row[l] + lane;
      const T al = static_cast<T>(s_al[j]), be = static_cast<T>(s_be[j]);
      const T pi = fma(be, a.p[row], a.u[row]);
      const T si = fma(be, a.s[row], a.w[row]);
      a.p[row] = pi;
      a.s[row] = si;
      a.x[row] = fma(al, pi, a.x[row]);
      const T ri = fma(-al, si, a.r[row]);
      a.r[row] = ri;
      a.u[row] = a.dinv[row] * ri;
    }
    if (!GBarSync(a.bar, epoch, &s_ok)) return;
    phase_b(false);
    if (!GBarSync(a.bar, epoch, &s_ok)) return;
  }
}

// Row count of every mesh's CSR rows: nnz[b] = rowptr[dof_off[b + 1]] - rowptr[dof_off[b]].
__global__ void MeshNnzKernel(int nb, const int64_t* __restrict__ dof_off, const int64_t* __restrict__ rowptr,
                              int64_t* __restrict__ nnz) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) nnz[b] = rowptr[dof_off[b + 1]] - rowptr[dof_off[b]];
}

// Per-mesh sums of chunk partials on the host (chunk order).
void MeshSums(lfg_batch* B, const double* dev_part, std::vector<double>& out) {
  std::vector<double> h(B->nchunks);
  LFG_CUDA(cudaMemcpyAsync(h.data(), dev_part, B->nchunks * sizeof(double), cudaMemcpyDeviceToHost, B->ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(B->ctx->stream));
  out.assign(B->nb, 0.0);
  for (int b = 0; b < B->nb; ++b)
    for (int64_t c = B->h_mesh_chunk_off[b]; c < B->h_mesh_chunk_off[b + 1]; ++c) out[b] += h[c];
}

template <class T>
struct BState {
  DevBuf r, z, p, q, part, ms;
};

template <class T>
void BAlloc(lfg_ctx* ctx, int64_t n, int64_t nch, int nb, BState<T>& S) {
  cudaStream_t s = ctx->stream;
  S.r.alloc(n * sizeof(T), s);
  S.z.alloc(n * sizeof(T), s);
  S.p.alloc(n * sizeof(T), s);
  S.q.alloc(n * sizeof(T), s);
  S.part.alloc(2 * nch * sizeof(double), s);
  S.ms.alloc(nb * sizeof(MeshScal), s);
  LFG_CUDA(cudaMemsetAsync(S.ms.p, 0, nb * sizeof(MeshScal), s));
}

// rr of every mesh (from the device scalars).
void MeshRR(lfg_batch* B, const DevBuf& ms, std::vector<double>& out) {
  std::vector<MeshScal> h(B->nb);
  LFG_CUDA(cudaMemcpyAsync(h.data(), ms.p, B->nb * sizeof(MeshScal), cudaMemcpyDeviceToHost, B->ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(B->ctx->stream));
  out.resize(B->nb);
  for (int b = 0; b < B->nb; ++b) out[b] = h[b].rr;
}

// `body` batched PCG iterations (even: the rz slots alternate) captured in a
// CUDA graph; frozen meshes are skipped by every kernel.
template <class T>
void BCapture(lfg_batch* B, lfg_csr* A, const T* sval, const T* rowsum, const T* dinv, T* x, BState<T>& S,
              const Chunks& C, DevBuf& frozen_d, int body, cudaGraph_t& graph, cudaGraphExec_t& exec) {
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  const int grid = static_cast<int>(std::min<int64_t>(C.nchunks, static_cast<int64_t>(ctx->num_sms) * 8));
  const Sell M{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>()};
  MeshScal* ms = S.ms.template as<MeshScal>();
  double* part = S.part.template as<double>();
  LFG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < body; ++k) {
    const int cur = k & 1;
    T* p = S.p.template as<T>();
    BDirectionKernel<T><<<grid, kPB, 0, s>>>(C, S.z.template as<T>(), p, frozen_d.as<int32_t>(), ms);
    BSpmvKernel<T><<<grid, kPB, 0, s>>>(C, M, sval, rowsum, p, S.q.template as<T>(), frozen_d.as<int32_t>(), cur,
                                        part, ms);
    BUpdateKernel<T><<<grid, kPB, 0, s>>>(C, dinv, p, S.q.template as<T>(), x, S.r.template as<T>(),
                                         S.z.template as<T>(), frozen_d.as<int32_t>(), cur, part, ms);
  }
  LFG_CUDA(cudaStreamEndCapture(s, &graph));
  LFG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
}

// Batched PCG in precision T on S.r (filled): per-mesh targets target_rr[b]
// (squared norms); meshes with frozen_h[b] start frozen.  Returns per-mesh
// iterations in it_out and final recursive rr in rr_out.
template <class T>
void BRunPcg(lfg_batch* B, lfg_csr* A, const T* sval, const T* rowsum, const T* dinv, T* x, BState<T>& S,
             const Chunks& C,
             const std::vector<double>& target_rr, std::vector<int32_t>& frozen_h, DevBuf& frozen_d, int max_it,
             int check_every, std::vector<int>& it_out, std::vector<double>& rr_out) {
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  const int grid = static_cast<int>(std::min<int64_t>(C.nchunks, static_cast<int64_t>(ctx->num_sms) * 8));
  MeshScal* ms = S.ms.template as<MeshScal>();
  double* part = S.part.template as<double>();
  LFG_CUDA(cudaMemcpyAsync(frozen_d.p, frozen_h.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  BStartKernel<T><<<grid, kPB, 0, s>>>(C, dinv, S.r.template as<T>(), S.z.template as<T>(), S.p.template as<T>(),
                                      frozen_d.as<int32_t>(), part, ms);
  LFG_LAUNCHED(ctx);
  std::vector<double> rr;
  MeshRR(B, S.ms, rr);
  it_out.assign(B->nb, 0);
  for (int b = 0; b < B->nb; ++b)
    if (!(rr[b] > target_rr[b])) frozen_h[b] = 1;
  LFG_CUDA(cudaMemcpyAsync(frozen_d.p, frozen_h.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  const int body = std::max(2, check_every + (check_every & 1));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  BCapture<T>(B, A, sval, rowsum, dinv, x, S, C, frozen_d, body, graph, exec);
  int it = 0;
  try {
    while (it < max_it) {
      int active = 0;
      for (int b = 0; b < B->nb; ++b) active += !frozen_h[b];
      if (!active) break;
      LFG_CUDA(cudaGraphLaunch(exec, s));
      CountLaunch(ctx, 3 * body);
      it += body;
      MeshRR(B, S.ms, rr);
      bool changed = false;
      for (int b = 0; b < B->nb; ++b)
        if (!frozen_h[b]) {
          it_out[b] = it;
          if (!(rr[b] > target_rr[b])) {
            frozen_h[b] = 1;
            changed = true;
          }
        }
      if (changed)
        LFG_CUDA(cudaMemcpyAsync(frozen_d.p, frozen_h.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
  } catch (...) {
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    throw;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  rr_out = rr;
}

// ---------------------------------------------------- grouped solver host
struct GBufs {
  DevBuf part, gs, bar, target, tabs, svec;
  std::vector<GMeshScal> gs_h;
  int grid = 0;
};

// nnz of every mesh's block of the CSR matrix.
std::vector<int64_t> MeshNnz(lfg_batch* B, lfg_csr* A) {
  lfg_ctx* ctx = B->ctx;
  DevBuf off, out;
  off.alloc((B->nb + 1) * sizeof(int64_t), ctx->stream);
  out.alloc(B->nb * sizeof(int64_t), ctx->stream);
  LFG_CUDA(cudaMemcpyAsync(off.p, B->dof_off.data(), (B->nb + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                           ctx->stream));
  MeshNnzKernel<<<(B->nb + 127) / 128, 128, 0, ctx->stream>>>(B->nb, off.as<int64_t>(), A->rowptr.as<int64_t>(),
                                                              out.as<int64_t>());
  LFG_LAUNCHED(ctx);
  std::vector<int64_t> h(B->nb);
  D2HSync(ctx, h.data(), out.p, B->nb * sizeof(int64_t));
  return h;
}

int64_t MeshLanesets(lfg_batch* B, int b) { return (B->dof_off[b + 1] - B->dof_off[b] + 31) / 32; }

// Meshes with want[b] packed into groups of at most `budget` bytes of solver
// data in precision T (padded matrix, Jacobi diagonal, row sums and the six
// work vectors), largest first; a mesh larger than the budget is a group of
// its own.  A group also holds at most max_ls lanesets.
template <class T>
std::vector<std::vector<int>> PackGroups(lfg_batch* B, const std::vector<int64_t>& nnz,
                                         const std::vector<int32_t>& want, double budget, int64_t max_ls) {
  std::vector<int> order;
  for (int b = 0; b < B->nb; ++b)
    if (want[b]) order.push_back(b);
  auto rows = [&](int b) { return B->dof_off[b + 1] - B->dof_off[b]; };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rows(a) > rows(b); });
  std::vector<std::vector<int>> groups;
  double used = 0.0;
  int64_t ls = 0;
  for (int b : order) {
    const double bytes = 1.1 * static_cast<double>(nnz[b]) * (4.0 + sizeof(T)) +
                         static_cast<double>(rows(b)) * 9.0 * sizeof(T);
    const int64_t nl = MeshLanesets(B, b);
    if (groups.empty() || used + bytes > budget || ls + nl > max_ls) {
      groups.emplace_back();
      used = 0.0;
      ls = 0;
    }
    groups.back().push_back(b);
    used += bytes;
    ls += nl;
  }
  return groups;
}

// Host copies of one group's device tables (lanesets, runs, block ranges).
struct GTabHost {
  std::vector<int64_t> ls_row;
  std::vector<int32_t> ls_n, ls_run, run_mesh, run_ls, run_m0, run_m1, blk_ls, blk_run;
};

// Lanesets of the group's meshes in group order, each block's contiguous
// range of them, and the runs (consecutive lanesets of one mesh within one
// block); uploaded into G.tabs.
GGroup UploadGroup(lfg_batch* B, const std::vector<int>& grp, int grid, GBufs& G, GTabHost& h) {
  h = GTabHost{};
  std::vector<int32_t> ls_mesh;
  for (int b : grp) {
    const int64_t r0 = B->dof_off[b], r1 = B->dof_off[b + 1];
    for (int64_t r = r0; r < r1; r += 32) {
      h.ls_row.push_back(r);
      h.ls_n.push_back(static_cast<int32_t>(std::min<int64_t>(32, r1 - r)));
      ls_mesh.push_back(b);
    }
  }
  const int64_t nl = static_cast<int64_t>(h.ls_row.size());
  if (nl > static_cast<int64_t>(kGMaxLs) * grid) Fail(LFG_UNSUPPORTED, "batched PCG: a group exceeds the cooperative grid");
  h.ls_run.resize(nl);
  h.blk_ls.resize(grid + 1);
  h.blk_run.resize(grid + 1);
  for (int k = 0; k <= grid; ++k) h.blk_ls[k] = static_cast<int32_t>(nl * k / grid);
  for (int k = 0; k < grid; ++k) {
    h.blk_run[k] = static_cast<int32_t>(h.run_mesh.size());
    for (int32_t l = h.blk_ls[k]; l < h.blk_ls[k + 1]; ++l) {
      if (l == h.blk_ls[k] || ls_mesh[l] != ls_mesh[l - 1]) {
        h.run_mesh.push_back(ls_mesh[l]);
        h.run_ls.push_back(l);
      }
      h.ls_run[l] = static_cast<int32_t>(h.run_mesh.size()) - 1;
    }
  }
  const int nrun = static_cast<int>(h.run_mesh.size());
  h.blk_run[grid] = nrun;
  h.run_ls.push_back(static_cast<int32_t>(nl));
  h.run_m0.resize(nrun);
  h.run_m1.resize(nrun);
  for (int q = 0; q < nrun;) {  // runs of one mesh are consecutive
    int e = q;
    while (e < nrun && h.run_mesh[e] == h.run_mesh[q]) ++e;
    for (int t = q; t < e; ++t) {
      h.run_m0[t] = q;
      h.run_m1[t] = e;
    }
    q = e;
  }
  // one buffer: the int64 laneset rows, then the int32 tables
  std::vector<int32_t> t32;
  auto add = [&](const std::vector<int32_t>& v) { t32.insert(t32.end(), v.begin(), v.end()); };
  add(h.ls_n);
  add(h.ls_run);
  add(h.run_mesh);
  add(h.run_ls);
  add(h.run_m0);
  add(h.run_m1);
  add(h.blk_ls);
  add(h.blk_run);
  const size_t bytes = static_cast<size_t>(nl) * 8 + t32.size() * 4;
  if (G.tabs.bytes < bytes) G.tabs.alloc(bytes, B->ctx->stream);
  LFG_CUDA(cudaMemcpyAsync(G.tabs.p, h.ls_row.data(), nl * 8, cudaMemcpyHostToDevice, B->ctx->stream));
  int32_t* d32 = reinterpret_cast<int32_t*>(static_cast<char*>(G.tabs.p) + nl * 8);
  LFG_CUDA(cudaMemcpyAsync(d32, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice, B->ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(B->ctx->stream));  // t32 is a local
  GGroup g;
  g.ls_row = static_cast<const int64_t*>(G.tabs.p);
  const int32_t* q = d32;
  g.ls_n = q;
  q += nl;
  g.ls_run = q;
  q += nl;
  g.run_mesh = q;
  q += nrun;
  g.run_ls = q;
  q += nrun + 1;
  g.run_m0 = q;
  q += nrun;
  g.run_m1 = q;
  q += nrun;
  g.blk_ls = q;
  q += grid + 1;
  g.blk_run = q;
  return g;
}

// Grouped PCG over `groups`: per group one (re)start of all its meshes, then
// cooperative launches of `body` iterations until every mesh of the group is
// frozen or max_it; after every launch `after(group, iterations)` runs with
// G.gs_h read back and returns true when it selected meshes (`sel`) to restart
// at the next launch (it uploads gs itself then).  `base` carries the vectors
// and operators; it_out[b] = iterations done by mesh b.
template <class T, class After>
void GRun(lfg_batch* B, GArgs<T> base, const int32_t* sel, GBufs& G, const std::vector<std::vector<int>>& groups,
          int max_it, int body, After after, std::vector<int>& it_out) {
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  GTabHost h;
  for (const std::vector<int>& grp : groups) {
    if (grp.empty()) continue;
    GArgs<T> ga = base;
    ga.g = UploadGroup(B, grp, G.grid, G, h);
    LFG_CUDA(cudaMemsetAsync(G.gs.p, 0, B->nb * sizeof(GMeshScal), s));
    ga.part = G.part.as<double>();
    ga.gs = G.gs.as<GMeshScal>();
    ga.target = G.target.as<double>();
    ga.bar = G.bar.as<GridBar>();
    ga.start = 1;
    ga.sel = nullptr;
    int i0 = 0;
    while (true) {
      ga.i0 = i0;
      ga.iters = std::min(body, max_it - i0);
      LFG_CUDA(cudaMemsetAsync(G.bar.p, 0, sizeof(GridBar), s));
      void* args[] = {&ga};
      LFG_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&BGroupCgKernel<T>), dim3(G.grid),
                                           dim3(kGThreads), args, 0, s));
      CountLaunch(ctx, 1);
      i0 += ga.iters;
      GridBar bar{};
      LFG_CUDA(cudaMemcpyAsync(&bar, G.bar.p, sizeof(GridBar), cudaMemcpyDeviceToHost, s));
      D2HSync(ctx, G.gs_h.data(), G.gs.p, B->nb * sizeof(GMeshScal));
      if (bar.err) Fail(LFG_CUDA_ERROR, "batched PCG: a grid barrier of the grouped solver timed out");
      const bool restart = after(grp, i0);
      ga.start = restart ? 1 : 0;
      ga.sel = restart ? sel : nullptr;
      int active = 0;
      for (int b : grp) active += !G.gs_h[b].frozen;
      if (!active || i0 >= max_it) break;
    }
    for (int b : grp) it_out[b] = G.gs_h[b].it;
  }
}

// Occupancy-sized cooperative grid (at most kGMinBlocks blocks per SM).
template <class T>
int GGrid(lfg_ctx* ctx) {
  int per_sm = 0;
  LFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, BGroupCgKernel<T>, kGThreads, 0));
  return ctx->num_sms * std::min(per_sm, kGMinBlocks);
}

template <class T>
void GAlloc(lfg_batch* B, int64_t n, GBufs& G) {
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  G.grid = GGrid<T>(ctx);
  if (G.grid < ctx->num_sms) Fail(LFG_CUDA_ERROR, "grouped PCG kernel cannot be resident");
  G.part.alloc(3 * static_cast<size_t>(kGMaxLs) * G.grid * sizeof(double), s);
  G.gs.alloc(B->nb * sizeof(GMeshScal), s);
  G.bar.alloc(sizeof(GridBar), s);
  G.target.alloc(B->nb * sizeof(double), s);
  G.svec.alloc(n * sizeof(T), s);
  G.gs_h.assign(B->nb, GMeshScal{});
}

// Chunks of `rows` rows, never straddling two meshes.
void BuildChunks(lfg_batch* B, int rows) {
  if (B->chunk_rows == rows) return;
  lfg_ctx* ctx = B->ctx;
  const int n = B->nb;
  std::vector<int32_t> cm;
  std::vector<int64_t> cs, mc(n + 1, 0);
  for (int b = 0; b < n; ++b) {
    mc[b] = static_cast<int64_t>(cm.size());
    for (int64_t r = B->dof_off[b]; r < B->dof_off[b + 1]; r += rows) {
      cm.push_back(b);
      cs.push_back(r);
    }
  }
  mc[n] = static_cast<int64_t>(cm.size());
  cs.push_back(B->dof_off[n]);
  B->nchunks = static_cast<int64_t>(cm.size());
  B->h_mesh_chunk_off = mc;
  B->chunk_mesh.alloc(std::max<size_t>(cm.size(), 1) * sizeof(int32_t), ctx->stream);
  B->chunk_start.alloc(cs.size() * sizeof(int64_t), ctx->stream);
  B->mesh_chunk_off.alloc(mc.size() * sizeof(int64_t), ctx->stream);
  if (!cm.empty())
    LFG_CUDA(cudaMemcpyAsync(B->chunk_mesh.p, cm.data(), cm.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             ctx->stream));
  LFG_CUDA(cudaMemcpyAsync(B->chunk_start.p, cs.data(), cs.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                           ctx->stream));
  LFG_CUDA(cudaMemcpyAsync(B->mesh_chunk_off.p, mc.data(), mc.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                           ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));  // the host vectors above are temporaries
  B->chunk_rows = rows;
}

// The autotuner's probe vectors: r = 1, x = 0 on every row.
template <class T>
__global__ void BFillKernel(int64_t n, T* __restrict__ r, T* __restrict__ x) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    r[i] = T(1);
    x[i] = T(0);
  }
}

// The batched PCG's autotuner: for each candidate number of rows per chunk
// (the work of one block between reductions), time `body` iterations of
// all blocks in precision T on scratch vectors and keep the candidate with
// the most row-iterations per second.
template <class T>
void TuneChunks(lfg_batch* B, lfg_csr* A, const T* sval, const T* rowsum, const T* dinv, int check) {
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  const int pi = sizeof(T) == 8 ? 0 : 1;
  const int64_t n = B->dof_off[B->nb];
  const int body = std::max(2, check + (check & 1));
  double best = -1.0;
  for (int rows : {512, 1024, 2048, 4096}) {
    BuildChunks(B, rows);
    Chunks C{B->chunk_mesh.as<int32_t>(), B->chunk_start.as<int64_t>(), B->mesh_chunk_off.as<int64_t>(), B->nchunks};
    const int grid = static_cast<int>(std::min<int64_t>(C.nchunks, static_cast<int64_t>(ctx->num_sms) * 8));
    BState<T> S;
    BAlloc(ctx, n, C.nchunks, B->nb, S);
    DevBuf xs, frozen;
    xs.alloc(n * sizeof(T), s);
    frozen.alloc(B->nb * sizeof(int32_t), s);
    LFG_CUDA(cudaMemsetAsync(frozen.p, 0, B->nb * sizeof(int32_t), s));
    const Sell M{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>()};
    MeshScal* ms = S.ms.template as<MeshScal>();
    double* part = S.part.template as<double>();
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    LFG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < body; ++k) {
      const int cur = k & 1;
      T* p = S.p.template as<T>();
      BDirectionKernel<T><<<grid, kPB, 0, s>>>(C, S.z.template as<T>(), p, frozen.as<int32_t>(), ms);
      BSpmvKernel<T><<<grid, kPB, 0, s>>>(C, M, sval, rowsum, p, S.q.template as<T>(), frozen.as<int32_t>(), cur,
                                          part, ms);
      BUpdateKernel<T><<<grid, kPB, 0, s>>>(C, dinv, p, S.q.template as<T>(), xs.as<T>(), S.r.template as<T>(),
                                           S.z.template as<T>(), frozen.as<int32_t>(), cur, part, ms);
    }
    LFG_CUDA(cudaStreamEndCapture(s, &graph));
    float ms_t = 0.f;
    try {
      LFG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
      for (int pass = 0; pass < 2; ++pass) {  // pass 0 warms the caches and the graph
        BFillKernel<T><<<GridFor(ctx, n, 256), 256, 0, s>>>(n, S.r.template as<T>(), xs.as<T>());
        BStartKernel<T><<<grid, kPB, 0, s>>>(C, dinv, S.r.template as<T>(), S.z.template as<T>(),
                                            S.p.template as<T>(), frozen.as<int32_t>(), part, ms);
        LFG_CUDA(cudaEventRecord(ctx->t0, s));
        LFG_CUDA(cudaGraphLaunch(exec, s));
        LFG_CUDA(cudaEventRecord(ctx->t1, s));
        LFG_CUDA(cudaEventSynchronize(ctx->t1));
        LFG_CUDA(cudaEventElapsedTime(&ms_t, ctx->t0, ctx->t1));
      }
    } catch (...) {
      if (exec) cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    CountLaunch(ctx, 4 + 6 * body);
    const double rate = static_cast<double>(n) * body / (ms_t * 1e-3);
    if (rate > best) {
      best = rate;
      B->solve_chunk_rows[pi] = rows;
    }
  }
  B->solve_rate[pi] = best;
  B->solve_tuned[pi] = true;
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_batch_create(lfg_ctx* ctx, int32_t n, lfg_space* const* spaces, lfg_batch** out) {
  LFG_API_BEGIN(ctx)
  if (!out || n <= 0 || !spaces) Fail(LFG_INVALID_ARG, "lfg_batch_create: bad argument");
  auto* B = new lfg_batch;
  try {
    B->ref.Set(ctx);
    B->ctx = ctx;
    B->nb = n;
    B->spaces.assign(spaces, spaces + n);
    B->dof_off.assign(n + 1, 0);
    B->cell_off.assign(n + 1, 0);
    B->trip_off.assign(n + 1, 0);
    std::vector<BatchMesh> hm(n);
    for (int b = 0; b < n; ++b) {
      lfg_space* sp = spaces[b];
      if (!sp || sp->mesh->ctx != ctx) Fail(LFG_INVALID_ARG, "space " + std::to_string(b) + " is null or on another context");
      if (sp->degree < 1) Fail(LFG_UNSUPPORTED, "batched assembly needs Lagrangian spaces");
      if (sp->mesh->nquad) Fail(LFG_UNSUPPORTED, "batched assembly supports triangular meshes");
      B->dof_off[b + 1] = B->dof_off[b] + sp->num_dofs;
      B->cell_off[b + 1] = B->cell_off[b] + sp->mesh->nc;
      B->trip_off[b + 1] = B->trip_off[b] + sp->num_triplets;
      B->max_degree = std::max(B->max_degree, sp->degree);
      BatchMesh& m = hm[b];
      m.xy = sp->mesh->xy.as<double2>();
      m.cells = sp->mesh->cell_nodes.as<int4>();
      m.cell_dofs = sp->cell_dofs.as<int32_t>();
      m.tri_offset = sp->tri_offset.as<int64_t>();
      m.n_cell = sp->n_cell;
      m.degree = sp->degree;
      m.ncells = sp->mesh->nc;
      m.dof_off = B->dof_off[b];
      m.cell_off = B->cell_off[b];
      m.trip_off = B->trip_off[b];
    }
    if (B->dof_off[n] >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "batch has more than 2^31 dofs");
    B->meshes.alloc(n * sizeof(BatchMesh), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(B->meshes.p, hm.data(), n * sizeof(BatchMesh), cudaMemcpyHostToDevice, ctx->stream));
    BuildChunks(B, kChunk);
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    delete B;
    throw;
  }
  *out = B;
  LFG_API_END
}

lfg_status lfg_batch_destroy(lfg_batch* B) {
  if (!B) return LFG_INVALID_ARG;
  cudaSetDevice(B->ctx->device);
  delete B;
  return LFG_OK;
}

lfg_status lfg_batch_info(const lfg_batch* B, int32_t* n, int64_t* dofs, int64_t* cells, int64_t* trips) {
  if (!B) return LFG_INVALID_ARG;
  if (n) *n = B->nb;
  if (dofs) *dofs = B->dof_off[B->nb];
  if (cells) *cells = B->cell_off[B->nb];
  if (trips) *trips = B->trip_off[B->nb];
  return LFG_OK;
}

lfg_status lfg_batch_offsets(const lfg_batch* B, int64_t* dof, int64_t* cell, int64_t* trip) {
  if (!B) return LFG_INVALID_ARG;
  for (int b = 0; b <= B->nb; ++b) {
    if (dof) dof[b] = B->dof_off[b];
    if (cell) cell[b] = B->cell_off[b];
    if (trip) trip[b] = B->trip_off[b];
  }
  return LFG_OK;
}

lfg_status lfg_batch_tuning(const lfg_batch* B, int32_t* threads, int32_t* ctas, double* ms) {
  if (!B) return LFG_INVALID_ARG;
  if (threads) *threads = B->tuned ? B->threads : 0;
  if (ctas) *ctas = B->tuned ? B->ctas_per_sm : 0;
  if (ms) *ms = B->best_ms;
  return LFG_OK;
}

lfg_status lfg_batch_solve_tuning(const lfg_batch* B, int32_t precision, int32_t* chunk_rows,
                                  double* row_iterations_per_s) {
  if (!B || (precision != LFG_SOLVE_FP64 && precision != LFG_SOLVE_MIXED)) return LFG_INVALID_ARG;
  const int pi = precision == LFG_SOLVE_MIXED ? 1 : 0;
  if (chunk_rows) *chunk_rows = B->solve_tuned[pi] ? B->solve_chunk_rows[pi] : 0;
  if (row_iterations_per_s) *row_iterations_per_s = B->solve_tuned[pi] ? B->solve_rate[pi] : 0.0;
  return LFG_OK;
}

lfg_status lfg_batch_set_solve_groups(lfg_batch* B, double group_bytes) {
  if (!B) return LFG_INVALID_ARG;
  LFG_API_BEGIN(B->ctx)
  if (!(group_bytes >= 0.0)) Fail(LFG_INVALID_ARG, "group_bytes must be >= 0");
  B->solve_group_bytes = group_bytes;
  LFG_API_END
}

lfg_status lfg_batch_solve_groups(const lfg_batch* B, double* group_bytes) {
  if (!B || !group_bytes) return LFG_INVALID_ARG;
  *group_bytes = B->solve_group_bytes;
  return LFG_OK;
}

lfg_status lfg_batch_set_solve_chunk_rows(lfg_batch* B, int32_t precision, int32_t chunk_rows) {
  if (!B) return LFG_INVALID_ARG;
  LFG_API_BEGIN(B->ctx)
  if (precision != LFG_SOLVE_FP64 && precision != LFG_SOLVE_MIXED) Fail(LFG_INVALID_ARG, "unknown solve precision");
  if (chunk_rows < 32 || chunk_rows > (1 << 20)) Fail(LFG_INVALID_ARG, "chunk_rows must be in [32, 2^20]");
  const int pi = precision == LFG_SOLVE_MIXED ? 1 : 0;
  B->solve_chunk_rows[pi] = chunk_rows;
  B->solve_rate[pi] = 0.0;
  B->solve_tuned[pi] = true;
  LFG_API_END
}

lfg_status lfg_batch_assemble_matrix_rd(lfg_batch* B, const lfg_rd_provider* pr, lfg_coo* coo) {
  if (!B) return LFG_INVALID_ARG;
  LFG_API_BEGIN(B->ctx)
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  if (!pr || !coo) Fail(LFG_INVALID_ARG, "lfg_batch_assemble_matrix_rd: null argument");
  const int64_t total = B->trip_off[B->nb];
  if (coo->rows < B->dof_off[B->nb] || coo->cols < B->dof_off[B->nb])
    Fail(LFG_INVALID_ARG, "COO matrix smaller than the batch");
  if (coo->size + total > coo->capacity) Fail(LFG_CAPACITY, "COO capacity too small for the batch");
  auto cell_const = [&](const lfg_coeff& c, const double*& data, double& value, const char* what) {
    data = nullptr;
    value = 0.0;
    if (c.kind == LFG_COEFF_CONSTANT) value = c.value;
    else if (c.kind == LFG_COEFF_PER_CELL) {
      if (!c.data_dev) Fail(LFG_INVALID_ARG, std::string(what) + ": null data");
      data = c.data_dev;
    } else if (c.kind != LFG_COEFF_ZERO) {
      Fail(LFG_UNSUPPORTED, std::string(what) + ": batched assembly takes constant or per-cell coefficients");
    }
  };
  BatchArgs A{};
  cell_const(pr->alpha, A.alpha, A.alpha_value, "alpha");
  cell_const(pr->gamma, A.gamma, A.gamma_value, "gamma");
  const bool mass = pr->gamma.kind != LFG_COEFF_ZERO;
  if (pr->qr_degree_tria < 0) Fail(LFG_MISSING_RULE, "no quadrature rule for triangles");
  // tables per degree (rule: default 2p or the given degree)
  std::vector<float> hdf;
  std::vector<double> h64;
  DevBuf tabs;
  {
    std::vector<std::pair<size_t, size_t>> offs(4, {0, 0});
    std::vector<unsigned char> blob;
    for (int deg = 1; deg <= 3; ++deg) {
      const int rd = pr->qr_degree_tria > 0 ? pr->qr_degree_tria : 2 * deg;
      DfLayout dl;
      if (!BuildDfTables(false, deg, rd, hdf, dl)) Fail(LFG_UNSUPPORTED, "no quadrature rule of that degree");
      // FP64 folded R from the df32 pair (hi + lo): exact to the pair's precision
      h64.assign(dl.E * 4, 0.0);
      for (int q = 0; q < dl.E * 4; ++q)
        h64[q] = static_cast<double>(hdf[2 * (dl.off_R + q)]) + static_cast<double>(hdf[2 * (dl.off_R + q) + 1]);
      const size_t o1 = blob.size();
      const size_t bytes_df = dl.E * 4 * 2 * sizeof(float);
      blob.resize(o1 + bytes_df);
      std::memcpy(blob.data() + o1, hdf.data() + 2 * dl.off_R, bytes_df);
      const size_t o2 = (blob.size() + 15) & ~size_t(15);
      blob.resize(o2 + h64.size() * sizeof(double));
      std::memcpy(blob.data() + o2, h64.data(), h64.size() * sizeof(double));
      blob.resize((blob.size() + 15) & ~size_t(15));
      offs[deg] = {o1, o2};
    }
    tabs.alloc(blob.size(), s);
    LFG_CUDA(cudaMemcpyAsync(tabs.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, s));
    for (int deg = 1; deg <= 3; ++deg) {
      A.tabs[deg] = reinterpret_cast<const f2*>(tabs.as<unsigned char>() + offs[deg].first);
      A.tabs64[deg] = reinterpret_cast<const double*>(tabs.as<unsigned char>() + offs[deg].second);
    }
  }
  A.meshes = B->meshes.as<BatchMesh>();
  A.nb = B->nb;
  A.out = coo->d + coo->size;
  A.fallback = reinterpret_cast<unsigned long long*>(StatusWord(ctx) + 12);
  const size_t stage = StagePerCell(B->max_degree);
  auto kernel = mass ? BatchAssembleKernel<true> : BatchAssembleKernel<false>;
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(kMaxBatchThreads * stage)));
  DevBuf prefix;
  prefix.alloc((B->nb + 1) * sizeof(int64_t), s);
  auto launch = [&](int threads, int ctas) {
    std::vector<int64_t> tp(B->nb + 1, 0);
    for (int b = 0; b < B->nb; ++b)
      tp[b + 1] = tp[b] + (B->spaces[b]->mesh->nc + threads - 1) / threads;
    LFG_CUDA(cudaMemcpyAsync(prefix.p, tp.data(), tp.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    A.tile_prefix = prefix.as<int64_t>();
    A.total_tiles = tp[B->nb];
    const size_t smem = threads * stage;
    const int64_t grid = std::min<int64_t>(A.total_tiles, static_cast<int64_t>(ctx->num_sms) * ctas);
    kernel<<<static_cast<unsigned>(std::max<int64_t>(grid, 1)), threads, smem, s>>>(A);
    LFG_LAUNCHED(ctx);
  };
  if (!B->tuned) {
    // autotuner: time every (threads per CTA, CTAs per SM) candidate once
    double best = 1e30;
    for (int threads : {64, 128, 256}) {
      int occ = 0;
      LFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, threads * stage));
      for (int ctas : {std::max(occ, 1), std::max(occ / 2, 1), std::max(2 * occ, 1)}) {
        launch(threads, ctas);  // warm
        LFG_CUDA(cudaEventRecord(ctx->t0, s));
        launch(threads, ctas);
        LFG_CUDA(cudaEventRecord(ctx->t1, s));
        LFG_CUDA(cudaEventSynchronize(ctx->t1));
        float ms = 0.f;
        LFG_CUDA(cudaEventElapsedTime(&ms, ctx->t0, ctx->t1));
        if (ms < best) {
          best = ms;
          B->threads = threads;
          B->ctas_per_sm = ctas;
        }
      }
    }
    B->best_ms = best;
    B->tuned = true;
  }
  {
    ProfScope prof(ctx, "batch_assemble");
    launch(B->threads, B->ctas_per_sm);
  }
  coo->size += total;
  LFG_API_END
}

lfg_status lfg_batch_assemble_vector_load(lfg_batch* B, const lfg_load_provider* pr, double* bvec) {
  if (!B) return LFG_INVALID_ARG;
  LFG_API_BEGIN(B->ctx)
  if (!pr || !bvec) Fail(LFG_INVALID_ARG, "lfg_batch_assemble_vector_load: null argument");
  if (pr->f.kind == LFG_COEFF_NODAL_O1) Fail(LFG_UNSUPPORTED, "batched load: nodal coefficients are not supported");
  for (int b = 0; b < B->nb; ++b) {
    lfg_load_provider p = *pr;
    if (p.f.kind == LFG_COEFF_PER_CELL) p.f.data_dev = pr->f.data_dev + B->cell_off[b];
    const lfg_status st = lfg_assemble_vector_load(B->spaces[b], &p, bvec + B->dof_off[b]);
    if (st != LFG_OK) Fail(st, B->ctx->last_error);
  }
  LFG_API_END
}

lfg_status lfg_batch_boundary_dof_flags(lfg_batch* B, uint8_t* flags) {
  if (!B) return LFG_INVALID_ARG;
  LFG_API_BEGIN(B->ctx)
  if (!flags) Fail(LFG_INVALID_ARG, "null flags");
  for (int b = 0; b < B->nb; ++b) {
    const lfg_status st = lfg_space_boundary_dof_flags(B->spaces[b], flags + B->dof_off[b]);
    if (st != LFG_OK) Fail(st, B->ctx->last_error);
  }
  LFG_API_END
}

lfg_status lfg_batch_solve_pcg(lfg_batch* B, lfg_csr* A, const double* bvec, double* x,
                               const lfg_solve_opts* opts, lfg_solve_stats* stats, lfg_solve_stats* per) {
  if (!B || !A) return LFG_INVALID_ARG;
  LFG_API_BEGIN(B->ctx)
  lfg_ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  if (!bvec || !x || !opts) Fail(LFG_INVALID_ARG, "lfg_batch_solve_pcg: null argument");
  const int64_t n = B->dof_off[B->nb];
  if (A->rows != n || A->cols != n) Fail(LFG_INVALID_ARG, "matrix size differs from the batch");
  if (A->nnz >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "solver needs nnz < 2^31");
  PrepareSolve(A);  // Jacobi diagonal, int32 row pointers, SELL-32 copy
  const bool mixed = opts->precision == LFG_SOLVE_MIXED;
  if (mixed) EnsureFloatValues(A);  // FP32 SELL values and row sums
  bool grouped = B->solve_group_bytes > 0.0;
  if (grouped) {
    // every mesh must fit one cooperative grid (at most kGMaxLs lanesets per block)
    const int64_t max_ls = static_cast<int64_t>(kGMaxLs) * (mixed ? GGrid<float>(ctx) : GGrid<double>(ctx));
    for (int b = 0; b < B->nb && grouped; ++b) grouped = MeshLanesets(B, b) <= max_ls;
    if (grouped) BuildChunks(B, kChunk);
  }
  if (!grouped) {
    const int pi = mixed ? 1 : 0;
    const int chk = opts->check_every > 0 ? opts->check_every : 32;
    if (!B->solve_tuned[pi]) {
      if (mixed)
        TuneChunks<float>(B, A, A->sell_val32.as<float>(), A->rowsum32.as<float>(), A->dinv32.as<float>(), chk);
      else if (opts->precision == LFG_SOLVE_FP64)
        TuneChunks<double>(B, A, A->sell_val.as<double>(), nullptr, A->dinv.as<double>(), chk);
    }
    BuildChunks(B, B->solve_chunk_rows[pi]);
  }
  Chunks C{B->chunk_mesh.as<int32_t>(), B->chunk_start.as<int64_t>(), B->mesh_chunk_off.as<int64_t>(), B->nchunks};
  const int grid = static_cast<int>(std::min<int64_t>(C.nchunks, static_cast<int64_t>(ctx->num_sms) * 8));
  const int check = opts->check_every > 0 ? opts->check_every : 32;
  const int max_it = opts->max_iterations > 0 ? opts->max_iterations : 100000;
  const double rtol = opts->rtol > 0 ? opts->rtol : 1e-10;
  BState<double> S;
  BAlloc(ctx, n, C.nchunks, B->nb, S);
  DevBuf frozen;
  frozen.alloc(B->nb * sizeof(int32_t), s);
  std::vector<double> bb, rr;
  BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(), nullptr,
                                      bvec, S.r.as<double>(), S.part.as<double>());
  LFG_LAUNCHED(ctx);
  MeshSums(B, S.part.as<double>(), bb);
  BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(), x, bvec,
                                      S.r.as<double>(), S.part.as<double>());
  LFG_LAUNCHED(ctx);
  MeshSums(B, S.part.as<double>(), rr);
  std::vector<double> target(B->nb);
  for (int b = 0; b < B->nb; ++b) target[b] = rtol * rtol * bb[b];
  std::vector<int32_t> frozen_h(B->nb, 0);
  std::vector<int> its(B->nb, 0), refinements(B->nb, 0);
  const int body = std::max(2, check + (check & 1));
  if (opts->precision == LFG_SOLVE_FP64) {
    std::vector<int> it1;
    std::vector<double> rr1;
    if (grouped) {
      GBufs G;
      GAlloc<double>(B, n, G);
      std::vector<int32_t> want(B->nb);
      for (int b = 0; b < B->nb; ++b) want[b] = rr[b] > target[b];
      const auto groups = PackGroups<double>(B, MeshNnz(B, A), want, B->solve_group_bytes,
                                             static_cast<int64_t>(G.grid) * kGMaxLs);
      LFG_CUDA(cudaMemcpyAsync(G.target.p, target.data(), B->nb * sizeof(double), cudaMemcpyHostToDevice, s));
      std::vector<int> itg(B->nb, 0);
      GArgs<double> base{};
      base.M = Sell{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>()};
      base.val = A->sell_val.as<double>();
      base.dinv = A->dinv.as<double>();
      base.x = x;
      base.r = S.r.as<double>();
      base.u = S.z.as<double>();
      base.w = S.q.as<double>();
      base.p = S.p.as<double>();
      base.s = G.svec.as<double>();
      GRun<double>(B, base, nullptr, G, groups, max_it, body, [](const std::vector<int>&, int) { return false; },
                   itg);
      for (int b = 0; b < B->nb; ++b) {
        its[b] += itg[b];
        refinements[b] += itg[b] > 0;
      }
      BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(), x,
                                          bvec, S.r.as<double>(), S.part.as<double>());
      LFG_LAUNCHED(ctx);
      MeshSums(B, S.part.as<double>(), rr);
    }
    // restart on the true residual when the recursive one drifted (<= 4 times)
    for (int round = 0; round < 5; ++round) {
      std::vector<int32_t> fz(B->nb, 0);
      int active = 0;
      for (int b = 0; b < B->nb; ++b) {
        fz[b] = !(rr[b] > target[b]);
        active += !fz[b];
      }
      if (!active) break;
      BRunPcg<double>(B, A, A->sell_val.as<double>(), nullptr, A->dinv.as<double>(), x, S, C, target, fz, frozen, max_it, check,
                      it1, rr1);
      for (int b = 0; b < B->nb; ++b) {
        its[b] += it1[b];
        refinements[b] += it1[b] > 0;
      }
      BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(), x,
                                          bvec, S.r.as<double>(), S.part.as<double>());
      LFG_LAUNCHED(ctx);
      MeshSums(B, S.part.as<double>(), rr);
    }
  } else if (opts->precision == LFG_SOLVE_MIXED) {
    // Per mesh: FP32 PCG on r / ||r_0|| with residual replacement (the
    // single-system solver's scheme, lfg_solve_pcg): once a mesh's recursive
    // FP32 residual has dropped by `drop` since its last replacement (or
    // reaches its target), its FP32 correction goes into x in FP64, its true
    // residual is formed in FP64 and replaces the recursive one, and its CG
    // continues along the same direction.  Meshes whose FP32 recursion stops
    // tracking the FP64 residual finish in FP64 afterwards.
    BState<float> S32;
    BAlloc(ctx, n, C.nchunks, B->nb, S32);
    DevBuf d32, scale, sel, frozen32;
    d32.alloc(n * sizeof(float), s);
    scale.alloc(B->nb * sizeof(double), s);
    sel.alloc(B->nb * sizeof(int32_t), s);
    frozen32.alloc(B->nb * sizeof(int32_t), s);
    const double drop = opts->inner_rtol > 0 ? opts->inner_rtol * opts->inner_rtol : 1e-2;
    std::vector<double> sc(B->nb), t32(B->nb), ref32(B->nb, 1.0), rr_last(rr);
    std::vector<int32_t> fz(B->nb), failed(B->nb, 0), sl(B->nb), keep(B->nb);
    // replacements in a row that did not cut the FP64 residual by 4: two end
    // the block's FP32 phase (else a block whose FP32 solves keep claiming
    // convergence just above its target would restart without end)
    std::vector<int32_t> stalls(B->nb, 0);
    // Smallest FP32 residual of each block since its last replacement, and
    // the checks in a row without a new minimum: a block whose recursion
    // found no new minimum in four checks is replaced as well (CG residuals
    // are not monotone, and a recursion that has lost orthogonality can hover
    // above the drop threshold for good)
    std::vector<double> best32(B->nb, INFINITY);
    std::vector<int32_t> flat(B->nb, 0);
    auto flat_check = [&](int b, double r32) {
      if (r32 < best32[b]) {
        best32[b] = r32;
        flat[b] = 0;
      } else {
        ++flat[b];
      }
      return flat[b] >= 4;
    };
    auto reset_flat = [&](int b) {
      best32[b] = INFINITY;
      flat[b] = 0;
    };
    for (int b = 0; b < B->nb; ++b) {
      fz[b] = !(rr[b] > target[b]);
      sc[b] = rr[b] > 0 ? 1.0 / std::sqrt(rr[b]) : 1.0;
      t32[b] = target[b] * sc[b] * sc[b];
    }
    LFG_CUDA(cudaMemcpyAsync(scale.p, sc.data(), B->nb * sizeof(double), cudaMemcpyHostToDevice, s));
    if (grouped) {
      GBufs G;
      GAlloc<float>(B, n, G);
      std::vector<int32_t> want(B->nb), done(B->nb, 0), cont(B->nb);
      for (int b = 0; b < B->nb; ++b) want[b] = rr[b] > target[b];
      const auto groups = PackGroups<float>(B, MeshNnz(B, A), want, B->solve_group_bytes,
                                            static_cast<int64_t>(G.grid) * kGMaxLs);
      LFG_CUDA(cudaMemcpyAsync(G.target.p, t32.data(), B->nb * sizeof(double), cudaMemcpyHostToDevice, s));
      std::vector<int> itg(B->nb, 0);
      std::vector<double> rr_new;
      // after every launch: residual replacement for the meshes whose FP32
      // residual dropped by `drop` (or that the kernel stopped as converged);
      // the meshes that go on restart at the next launch (sel = cont)
      auto after = [&](const std::vector<int>& grp, int i_done) -> bool {
        int nsel = 0;
        for (int b = 0; b < B->nb; ++b) sl[b] = 0;
        for (int b : grp) {
          if (done[b]) continue;
          const GMeshScal& m = G.gs_h[b];
          if (!std::isfinite(m.rr)) {  // FP32 broke down: finish this block in FP64 from its x
            failed[b] = 1;
            done[b] = 1;
            G.gs_h[b].frozen = 1;
            continue;
          }
          sl[b] = m.frozen || !(m.rr >= drop * ref32[b]) || flat_check(b, m.rr) || i_done >= max_it;
          if (sl[b]) reset_flat(b);
          nsel += sl[b];
        }
        if (!nsel) {
          LFG_CUDA(cudaMemcpyAsync(G.gs.p, G.gs_h.data(), B->nb * sizeof(GMeshScal), cudaMemcpyHostToDevice, s));
          return false;
        }
        LFG_CUDA(cudaMemcpyAsync(sel.p, sl.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        BApplyKernel<<<grid, kPB, 0, s>>>(C, d32.as<float>(), scale.as<double>(), sel.as<int32_t>(), 1.0, x);
        LFG_LAUNCHED(ctx);
        BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                            x, bvec, S.r.as<double>(), S.part.as<double>(), sel.as<int32_t>());
        LFG_LAUNCHED(ctx);
        MeshSums(B, S.part.as<double>(), rr_new);
        int nrevert = 0, nkeep = 0;
        for (int b = 0; b < B->nb; ++b) {
          cont[b] = 0;
          if (!sl[b]) continue;
          refinements[b] += 1;
          const double claimed = G.gs_h[b].rr / (sc[b] * sc[b]);
          const bool progress = rr_new[b] < 0.25 * rr_last[b];
          stalls[b] = progress ? 0 : stalls[b] + 1;
          if (rr_new[b] <= target[b]) {
            rr[b] = rr_new[b];
            done[b] = 1;
            G.gs_h[b].frozen = 1;
          } else if ((!progress && !(rr_new[b] <= 16.0 * claimed)) || stalls[b] >= 2) {
            failed[b] = 1;
            done[b] = 1;
            G.gs_h[b].frozen = 1;
            if (!(rr_new[b] < rr_last[b])) {
              sl[b] = 2;
              ++nrevert;
            } else {
              rr[b] = rr_new[b];
            }
          } else {
            rr[b] = rr_last[b] = rr_new[b];
            ref32[b] = rr_new[b] * sc[b] * sc[b];
            if (i_done >= max_it) {
              done[b] = 1;
              G.gs_h[b].frozen = 1;
            } else {
              cont[b] = 1;
              ++nkeep;
              G.gs_h[b].frozen = 0;
              G.gs_h[b].fresh = i_done;  // restarts (beta = 0) at the next launch
            }
          }
        }
        if (nrevert) {
          for (int b = 0; b < B->nb; ++b) sl[b] = sl[b] == 2;
          LFG_CUDA(cudaMemcpyAsync(sel.p, sl.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
          BApplyKernel<<<grid, kPB, 0, s>>>(C, d32.as<float>(), scale.as<double>(), sel.as<int32_t>(), -1.0, x);
          LFG_LAUNCHED(ctx);
          BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                              A->val.as<double>(), x, bvec, S.r.as<double>(), S.part.as<double>(),
                                              sel.as<int32_t>());
          LFG_LAUNCHED(ctx);
          MeshSums(B, S.part.as<double>(), rr_new);
          for (int b = 0; b < B->nb; ++b)
            if (sl[b]) rr[b] = rr_new[b];
        }
        if (nkeep) LFG_CUDA(cudaMemcpyAsync(sel.p, cont.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        LFG_CUDA(cudaMemcpyAsync(G.gs.p, G.gs_h.data(), B->nb * sizeof(GMeshScal), cudaMemcpyHostToDevice, s));
        return nkeep > 0;
      };
      GArgs<float> base{};
      base.M = Sell{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>()};
      base.val = A->sell_val32.as<float>();
      base.rowsum = A->rowsum32.as<float>();
      base.dinv = A->dinv32.as<float>();
      base.x = d32.as<float>();
      base.r = S32.r.as<float>();
      base.u = S32.z.as<float>();
      base.w = S32.q.as<float>();
      base.p = S32.p.as<float>();
      base.s = G.svec.as<float>();
      base.r64 = S.r.as<double>();
      base.scale = scale.as<double>();
      GRun<float>(B, base, sel.as<int32_t>(), G, groups, max_it, body, after, itg);
      for (int b = 0; b < B->nb; ++b) its[b] += itg[b];
    } else {
    LFG_CUDA(cudaMemcpyAsync(frozen32.p, fz.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    BScaleKernel<<<grid, kPB, 0, s>>>(C, S.r.as<double>(), scale.as<double>(), S32.r.as<float>(), d32.as<float>());
    LFG_LAUNCHED(ctx);
    BStartKernel<float><<<grid, kPB, 0, s>>>(C, A->dinv32.as<float>(), S32.r.as<float>(), S32.z.as<float>(),
                                             S32.p.as<float>(), frozen32.as<int32_t>(), S32.part.as<double>(),
                                             S32.ms.as<MeshScal>());
    LFG_LAUNCHED(ctx);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BCapture<float>(B, A, A->sell_val32.as<float>(), A->rowsum32.as<float>(), A->dinv32.as<float>(), d32.as<float>(),
                    S32, C, frozen32, body, graph, exec);
    std::vector<double> rr32, rr_new;
    int it = 0;
    try {
      while (true) {
        int active = 0;
        for (int b = 0; b < B->nb; ++b) active += !fz[b];
        if (!active) break;
        LFG_CUDA(cudaGraphLaunch(exec, s));
        CountLaunch(ctx, 3 * body);
        it += body;
        MeshRR(B, S32.ms, rr32);
        int nsel = 0;
        for (int b = 0; b < B->nb; ++b) {
          sl[b] = 0;
          if (fz[b]) continue;
          its[b] += body;
          if (!std::isfinite(rr32[b])) {  // FP32 broke down: finish this block in FP64 from its x
            failed[b] = 1;
            fz[b] = 1;
            continue;
          }
          sl[b] = !(rr32[b] > t32[b]) || !(rr32[b] >= drop * ref32[b]) || flat_check(b, rr32[b]) || it >= max_it;
          if (sl[b]) reset_flat(b);
          nsel += sl[b];
        }
        if (!nsel) {
          LFG_CUDA(cudaMemcpyAsync(frozen32.p, fz.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
          continue;
        }
        LFG_CUDA(cudaMemcpyAsync(sel.p, sl.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        BApplyKernel<<<grid, kPB, 0, s>>>(C, d32.as<float>(), scale.as<double>(), sel.as<int32_t>(), 1.0, x);
        LFG_LAUNCHED(ctx);
        BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                            x, bvec, S.r.as<double>(), S.part.as<double>(), sel.as<int32_t>());
        LFG_LAUNCHED(ctx);
        MeshSums(B, S.part.as<double>(), rr_new);
        int nrevert = 0, nkeep = 0;
        for (int b = 0; b < B->nb; ++b) {
          keep[b] = 0;
          if (!sl[b]) continue;
          refinements[b] += 1;
          const double claimed = rr32[b] / (sc[b] * sc[b]);
          const bool progress = rr_new[b] < 0.25 * rr_last[b];
          stalls[b] = progress ? 0 : stalls[b] + 1;
          if (rr_new[b] <= target[b]) {
            rr[b] = rr_new[b];
            fz[b] = 1;
          } else if ((!progress && !(rr_new[b] <= 16.0 * claimed)) || stalls[b] >= 2) {
            failed[b] = 1;  // FP32 cannot resolve this block: finish it in FP64
            fz[b] = 1;
            if (!(rr_new[b] < rr_last[b])) {
              sl[b] = 2;  // take the correction back
              ++nrevert;
            } else {
              rr[b] = rr_new[b];
            }
          } else {
            rr[b] = rr_last[b] = rr_new[b];
            ref32[b] = rr_new[b] * sc[b] * sc[b];
            if (it >= max_it) {
              fz[b] = 1;
            } else {
              keep[b] = 1;
              ++nkeep;
            }
          }
        }
        if (nrevert) {
          for (int b = 0; b < B->nb; ++b) sl[b] = sl[b] == 2;
          LFG_CUDA(cudaMemcpyAsync(sel.p, sl.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
          BApplyKernel<<<grid, kPB, 0, s>>>(C, d32.as<float>(), scale.as<double>(), sel.as<int32_t>(), -1.0, x);
          LFG_LAUNCHED(ctx);
          BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                              A->val.as<double>(), x, bvec, S.r.as<double>(), S.part.as<double>(),
                                              sel.as<int32_t>());
          LFG_LAUNCHED(ctx);
          MeshSums(B, S.part.as<double>(), rr_new);
          for (int b = 0; b < B->nb; ++b)
            if (sl[b]) rr[b] = rr_new[b];
        }
        if (nkeep) {
          LFG_CUDA(cudaMemcpyAsync(sel.p, keep.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
          BReplaceKernel<<<grid, kPB, 0, s>>>(C, S.r.as<double>(), scale.as<double>(), A->dinv32.as<float>(),
                                             S32.r.as<float>(), S32.z.as<float>(), d32.as<float>(), sel.as<int32_t>(),
                                             S32.part.as<double>(), S32.ms.as<MeshScal>());
          LFG_LAUNCHED(ctx);
        }
        LFG_CUDA(cudaMemcpyAsync(frozen32.p, fz.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
      }
    } catch (...) {
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    }
    // blocks FP32 could not finish: FP64 PCG from their current iterate
    int nfailed = 0;
    for (int b = 0; b < B->nb; ++b) nfailed += failed[b] && rr[b] > target[b];
    if (nfailed) {
      std::vector<int> it1;
      std::vector<double> rr1, rr_new;
      for (int round = 0; round < 5; ++round) {
        std::vector<int32_t> f64(B->nb, 1);
        int act = 0;
        for (int b = 0; b < B->nb; ++b) {
          f64[b] = !(failed[b] && rr[b] > target[b]);
          act += !f64[b];
        }
        if (!act) break;
        std::vector<int32_t> only(B->nb);
        for (int b = 0; b < B->nb; ++b) only[b] = !f64[b];
        LFG_CUDA(cudaMemcpyAsync(sel.p, only.data(), B->nb * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                            x, bvec, S.r.as<double>(), S.part.as<double>(), sel.as<int32_t>());
        LFG_LAUNCHED(ctx);
        BRunPcg<double>(B, A, A->sell_val.as<double>(), nullptr, A->dinv.as<double>(), x, S, C, target, f64, frozen,
                        max_it, check, it1, rr1);
        BResidualKernel<<<grid, kPB, 0, s>>>(C, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                            x, bvec, S.r.as<double>(), S.part.as<double>(), sel.as<int32_t>());
        LFG_LAUNCHED(ctx);
        MeshSums(B, S.part.as<double>(), rr_new);
        bool progress = false;
        for (int b = 0; b < B->nb; ++b)
          if (only[b]) {
            its[b] += it1[b];
            refinements[b] += 1;
            progress = progress || rr_new[b] < 0.25 * rr[b];
            rr[b] = rr_new[b];
          }
        if (!progress) break;
      }
    }
  } else {
    Fail(LFG_INVALID_ARG, "unknown solve precision");
  }
  lfg_solve_stats tot{};
  tot.converged = 1;
  double worst = 0.0;
  for (int b = 0; b < B->nb; ++b) {
    lfg_solve_stats sb{};
    sb.iterations = its[b];
    sb.refinements = refinements[b];
    sb.rel_residual = bb[b] > 0 ? std::sqrt(rr[b] / bb[b]) : 0.0;
    sb.converged = bb[b] == 0 || sb.rel_residual <= rtol * 1.0000001;
    if (per) per[b] = sb;
    tot.iterations = std::max(tot.iterations, sb.iterations);
    tot.refinements = std::max(tot.refinements, sb.refinements);
    tot.converged = tot.converged && sb.converged;
    worst = std::max(worst, sb.rel_residual);
  }
  tot.rel_residual = worst;
  if (stats) *stats = tot;
  if (!tot.converged) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "batched PCG: not all blocks converged (worst rel. residual %.3e)", worst);
    Fail(LFG_NOT_CONVERGED, buf);
  }
  LFG_API_END
}

}  // extern "C"
