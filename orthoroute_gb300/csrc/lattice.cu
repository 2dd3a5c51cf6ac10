// A1: 3-D Manhattan lattice → CSR, built on the device in closed form.
//
// Row layout of node (x, y, z), sorted by destination id as the reference's
// structured sort leaves it (unified_pathfinder.py:935):
//   [via partners z' < z, ascending] [y-1] [x-1] [x+1] [y+1] [via partners z' > z]
// Lateral arcs exist only on lateral layers and only along the layer's axis
// (plus the other axis when wrong-way arcs are enabled).  A via partner is
// present when (x, y) is a legal site of that layer pair.
#include "common.cuh"

namespace {

constexpr int kMaxLayers = 64;
constexpr int kMaxPartners = 64 * 64;

struct LatticeConst {
  int nx, ny, nz;
  float lateral_cost, wrong_way_cost;
  unsigned char axis[kMaxLayers];
  int pptr[kMaxLayers + 1];
};

// The lattice description travels as a kernel argument and its via-partner
// tables live in the build workspace, so builds on different streams (jobs
// of a server) do not share state.
struct LatDev {
  LatticeConst h;
  const int* pz;
  const float* pcost;
  const int* psite;
};

__device__ __forceinline__ bool site_ok(int mode, int x, int y) {
  if (mode == 0) return true;
  if (mode == 1) return ((x + y) & 1) == 0;
  return (x % mode) == 0 && (y % mode) == 0;
}

// Number of arcs and (optionally) the row itself.
template <bool kWrite>
__device__ __forceinline__ int node_row(const LatDev& L, int64_t n, int32_t* idx, float* cost, unsigned char* lay,
                                        unsigned char* kind) {
  const int nx = L.h.nx, ny = L.h.ny;
  const int64_t plane = (int64_t)nx * ny;
  const int z = (int)(n / plane);
  const int64_t r = n - (int64_t)z * plane;
  const int y = (int)(r / nx);
  const int x = (int)(r - (int64_t)y * nx);
  int k = 0;
  const int p0 = L.h.pptr[z], p1 = L.h.pptr[z + 1];
  for (int p = p0; p < p1; ++p) {
    const int zz = L.pz[p];
    if (zz >= z) break;
    if (!site_ok(L.psite[p], x, y)) continue;
    if (kWrite) {
      idx[k] = (int32_t)((int64_t)zz * plane + r);
      cost[k] = L.pcost[p];
      lay[k] = (unsigned char)z;
      kind[k] = 1;
    }
    ++k;
  }
  const int ax = L.h.axis[z];
  if (ax != 0) {
    const bool ww = L.h.wrong_way_cost > 0.f;
    const bool h = (ax == 1) || ww;
    const bool v = (ax == 2) || ww;
    const float ch = (ax == 1) ? L.h.lateral_cost : L.h.wrong_way_cost;
    const float cv = (ax == 2) ? L.h.lateral_cost : L.h.wrong_way_cost;
    if (v && y > 0) {
      if (kWrite) { idx[k] = (int32_t)(n - nx); cost[k] = cv; lay[k] = (unsigned char)z; kind[k] = 0; }
      ++k;
    }
    if (h && x > 0) {
      if (kWrite) { idx[k] = (int32_t)(n - 1); cost[k] = ch; lay[k] = (unsigned char)z; kind[k] = 0; }
      ++k;
    }
    if (h && x + 1 < nx) {
      if (kWrite) { idx[k] = (int32_t)(n + 1); cost[k] = ch; lay[k] = (unsigned char)z; kind[k] = 0; }
      ++k;
    }
    if (v && y + 1 < ny) {
      if (kWrite) { idx[k] = (int32_t)(n + nx); cost[k] = cv; lay[k] = (unsigned char)z; kind[k] = 0; }
      ++k;
    }
  }
  for (int p = p0; p < p1; ++p) {
    const int zz = L.pz[p];
    if (zz <= z) continue;
    if (!site_ok(L.psite[p], x, y)) continue;
    if (kWrite) {
      idx[k] = (int32_t)((int64_t)zz * plane + r);
      cost[k] = L.pcost[p];
      lay[k] = (unsigned char)z;
      kind[k] = 1;
    }
    ++k;
  }
  return k;
}

__global__ void degree_kernel(LatDev L, int64_t N, int32_t* deg) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N;
       n += (int64_t)gridDim.x * blockDim.x)
    deg[n] = node_row<false>(L, n, nullptr, nullptr, nullptr, nullptr);
}

// Exclusive scan, 3 phases: per-tile sums, scan of tile sums (1 block), add.
constexpr int kScanTile = 1024;

__global__ void scan_tiles(const int32_t* in, int64_t N, int32_t* out, int32_t* tile_sums) {
  __shared__ int32_t s[kScanTile];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  const int t = threadIdx.x;
  const int64_t i = base + t;
  int32_t v = (i < N) ? in[i] : 0;
  s[t] = v;
  __syncthreads();
  for (int off = 1; off < kScanTile; off <<= 1) {
    int32_t a = (t >= off) ? s[t - off] : 0;
    __syncthreads();
    s[t] += a;
    __syncthreads();
  }
  if (i < N) out[i] = s[t] - v;  // exclusive within tile
  if (t == kScanTile - 1) tile_sums[blockIdx.x] = s[t];
}

__global__ void scan_tile_sums(int32_t* tile_sums, int64_t ntiles, int32_t* total) {
  // Single block, sequential over chunks of kScanTile.
  __shared__ int32_t s[kScanTile];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += kScanTile) {
    const int t = threadIdx.x;
    const int64_t i = base + t;
    int32_t v = (i < ntiles) ? tile_sums[i] : 0;
    s[t] = v;
    __syncthreads();
    for (int off = 1; off < kScanTile; off <<= 1) {
      int32_t a = (t >= off) ? s[t - off] : 0;
      __syncthreads();
      s[t] += a;
      __syncthreads();
    }
    if (i < ntiles) tile_sums[i] = carry + s[t] - v;
    __syncthreads();
    if (t == kScanTile - 1) carry += s[t];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_add(int32_t* out, int64_t N, const int32_t* tile_sums, const int32_t* total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= N;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i == N) out[N] = *total;
    else out[i] += tile_sums[i / kScanTile];
  }
}

__global__ void fill_kernel(LatDev L, int64_t N, const int32_t* indptr, int32_t* indices, float* cost,
                            unsigned char* lay, unsigned char* kind, int32_t* edge_src) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = indptr[n];
    const int k = node_row<true>(L, n, indices + b, cost + b, lay + b, kind + b);
    for (int j = 0; j < k; ++j) edge_src[b + j] = (int32_t)n;
  }
}

__global__ void rev_kernel(int64_t N, const int32_t* indptr, const int32_t* indices, int32_t* rev) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < N;
       u += (int64_t)gridDim.x * blockDim.x) {
    for (int32_t e = indptr[u]; e < indptr[u + 1]; ++e) {
      const int32_t v = indices[e];
      int32_t found = -1;
      for (int32_t f = indptr[v]; f < indptr[v + 1]; ++f)
        if (indices[f] == (int32_t)u) { found = f; break; }
      rev[e] = found;
    }
  }
}

// Fills the description; the partner tables are copied on `s` into dev_tab
// (3 * kMaxPartners words of the workspace).
int load_desc(const ogr_lattice_desc* d, int* dev_tab, cudaStream_t s, LatDev* out) {
  if (!d || d->nx < 1 || d->ny < 1 || d->nz < 1 || d->nz > kMaxLayers) return OGR_ERR_ARG;
  LatDev L{};
  LatticeConst& h = L.h;
  h.nx = d->nx; h.ny = d->ny; h.nz = d->nz;
  h.lateral_cost = d->lateral_cost;
  h.wrong_way_cost = d->wrong_way_cost;
  for (int z = 0; z < d->nz; ++z) h.axis[z] = d->layer_axis[z];
  for (int z = 0; z <= d->nz; ++z) h.pptr[z] = d->partner_ptr[z];
  const int np = d->partner_ptr[d->nz];
  if (np > kMaxPartners || np < 0) return OGR_ERR_ARG;
  L.pz = dev_tab;
  L.pcost = reinterpret_cast<const float*>(dev_tab + kMaxPartners);
  L.psite = dev_tab + 2 * kMaxPartners;
  if (np > 0) {
    OGR_CUDA_TRY(cudaMemcpyAsync(dev_tab, d->partner_z, np * sizeof(int), cudaMemcpyHostToDevice, s));
    OGR_CUDA_TRY(cudaMemcpyAsync(dev_tab + kMaxPartners, d->partner_cost, np * sizeof(float),
                                 cudaMemcpyHostToDevice, s));
    OGR_CUDA_TRY(cudaMemcpyAsync(dev_tab + 2 * kMaxPartners, d->partner_site, np * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
  }
  *out = L;
  return OGR_OK;
}

// Host mirror of the per-node arc count (for sizing).
int64_t host_num_edges(const ogr_lattice_desc* d) {
  const int64_t nx = d->nx, ny = d->ny;
  int64_t E = 0;
  for (int z = 0; z < d->nz; ++z) {
    const int ax = d->layer_axis[z];
    const bool ww = d->wrong_way_cost > 0.f;
    if (ax != 0) {
      if (ax == 1 || ww) E += 2 * ny * (nx - 1);
      if (ax == 2 || ww) E += 2 * nx * (ny - 1);
    }
    for (int p = d->partner_ptr[z]; p < d->partner_ptr[z + 1]; ++p) {
      const int mode = d->partner_site[p];
      int64_t sites = 0;
      if (mode == 0) sites = nx * ny;
      else {
        for (int64_t x = 0; x < nx; ++x)
          for (int64_t y = 0; y < ny; ++y)
            if (mode == 1 ? ((x + y) % 2 == 0) : (x % mode == 0 && y % mode == 0)) ++sites;
      }
      E += sites;
    }
  }
  return E;
}

}  // namespace

extern "C" int ogr_csr_num_edges(const ogr_lattice_desc* d, int64_t* num_edges) {
  if (!d || !num_edges || d->nz > kMaxLayers) return OGR_ERR_ARG;
  *num_edges = host_num_edges(d);
  return OGR_OK;
}

extern "C" size_t ogr_csr_workspace_bytes(const ogr_lattice_desc* d) {
  const int64_t N = (int64_t)d->nx * d->ny * d->nz;
  const int64_t tiles = (N + kScanTile - 1) / kScanTile;
  return (size_t)(N * 4 + tiles * 4 + 64) + 3 * sizeof(int) * kMaxPartners + 256;
}

extern "C" int ogr_csr_build(const ogr_lattice_desc* d, int32_t* indptr, int32_t* indices,
                             float* base_costs, uint8_t* edge_layer, uint8_t* edge_kind,
                             int32_t* edge_src, int32_t* rev, void* workspace,
                             size_t workspace_bytes, void* stream) {
  if (!d || d->nz > kMaxLayers || d->nz < 1) return OGR_ERR_ARG;
  const int64_t N = (int64_t)d->nx * d->ny * d->nz;
  if (N >= (int64_t)1 << 31) return OGR_ERR_ARG;
  const int64_t E = host_num_edges(d);
  if (E >= (int64_t)1 << 31) return OGR_ERR_ARG;
  if (workspace_bytes < ogr_csr_workspace_bytes(d) || !workspace) return OGR_ERR_CAPACITY;
  cudaStream_t s = ogr_stream(stream);
  int32_t* deg = reinterpret_cast<int32_t*>(workspace);
  const int64_t tiles = (N + kScanTile - 1) / kScanTile;
  int32_t* tile_sums = deg + N;
  int32_t* total = tile_sums + tiles;
  const size_t tab_off = ((size_t)(N * 4 + tiles * 4 + 64) + 255) & ~(size_t)255;
  LatDev L;
  const int rc = load_desc(d, reinterpret_cast<int*>((char*)workspace + tab_off), s, &L);
  if (rc != OGR_OK) return rc;
  degree_kernel<<<ogr_blocks(N, 256), 256, 0, s>>>(L, N, deg);
  scan_tiles<<<(unsigned)tiles, kScanTile, 0, s>>>(deg, N, indptr, tile_sums);
  scan_tile_sums<<<1, kScanTile, 0, s>>>(tile_sums, tiles, total);
  scan_add<<<ogr_blocks(N + 1, 256), 256, 0, s>>>(indptr, N, tile_sums, total);
  fill_kernel<<<ogr_blocks(N, 256), 256, 0, s>>>(L, N, indptr, indices, base_costs, edge_layer, edge_kind,
                                                  edge_src);
  if (rev) rev_kernel<<<ogr_blocks(N, 256), 256, 0, s>>>(N, indptr, indices, rev);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}
