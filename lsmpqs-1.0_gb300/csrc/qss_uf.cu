// qss_uf.cu -- 26-connected component labelling and trapped-phase masks on GB300.
//
// The reference labels {phi_bin == 1} with a serial union-find whose union
// rule always hangs the smaller root under the larger one
// (src/connectivity/connectivity.c:66-83), so every component ends up named
// by its LARGEST linear ghost-box index, and background is 0 (:201-214).
// That label is a property of the component, not of the visiting order, so a
// concurrent union-find that keeps the same rule (link the smaller root under
// the larger, by compare-and-swap on the root) produces identical labels:
//   1. per 8x8x8 tile, in shared memory: every foreground voxel unites with
//      its preceding neighbours inside the tile; parent[v] = the global index
//      of v's tile-local root (0 for background);
//   2. voxels on a tile face unite, in global memory, with their preceding
//      neighbours in other tiles (every adjacent pair is a preceding pair
//      from one side);
//   3. labels[v] = root(v), 0 for background.
// Every write to parent[] increases it (hooking a root under a larger root,
// or compressing a node to a larger ancestor), so parent[x] > x holds for
// every non-root, the pointer graph has no cycle and every walk ends; the
// walks still carry an iteration cap and set an error flag instead of
// spinning if the cap is ever reached.
#include "qss_kernels.cuh"

namespace qss {

namespace {

// longest pointer walk tolerated before a device-side error is flagged
constexpr int kWalkCap = 1 << 22;

__device__ __forceinline__ int find_root(int* parent, int x, int* err) {
  int r = x;
  int it = 0;
  while (true) {
    int p = __ldcg(parent + r);  // L2-coherent read: other blocks hook roots concurrently
    if (p == r) break;
    r = p;
    if (++it > kWalkCap) {
      *err |= ERR_UF_LIMIT;
      return r;
    }
  }
  // Path compression.  Only nodes below r are rewritten, and only upwards:
  // another thread may already have moved a node of this path above r, and
  // lowering it again (or walking past r) could close a cycle.
  int y = x;
  it = 0;
  while (y < r && it++ < kWalkCap) {
    const int p = __ldcg(parent + y);
    if (p < r) __stcg(parent + y, r);
    y = p;
  }
  return r;
}

__device__ __forceinline__ void unite(int* parent, int a, int b, int* err) {
  int ra = find_root(parent, a, err);
  int rb = find_root(parent, b, err);
  int it = 0;
  while (ra != rb) {
    if (ra > rb) {
      int t = ra;
      ra = rb;
      rb = t;
    }
    const int old = atomicCAS(&parent[ra], ra, rb);  // hang the smaller root under the larger
    if (old == ra) return;
    ra = find_root(parent, old, err);
    rb = find_root(parent, rb, err);
    if (++it > kWalkCap) {
      *err |= ERR_UF_LIMIT;
      return;
    }
  }
}

// Tiles of 8 x 8 x 8 voxels: inside a tile the union-find runs in shared
// memory (same rule: the smaller root is hung under the larger, so the local
// root is the tile component's largest index, and the local order of a tile
// is the global linear order restricted to it); then every voxel's global
// parent is the global index of its local root (depth 1), and only the
// adjacencies that cross a tile face are united in global memory.
constexpr int kTile = 8;
constexpr int kTileN = kTile * kTile * kTile;
constexpr int kTileThreads = 256;

__device__ __forceinline__ int lfind(int* lp, int x, int* err) {
  int r = x;
  int it = 0;
  while (true) {
    const int p = lp[r];
    if (p == r) break;
    r = p;
    if (++it > kTileN) {
      *err |= ERR_UF_LIMIT;
      return r;
    }
  }
  int y = x;
  it = 0;
  while (y < r && it++ < kTileN) {  // compression upwards only (see find_root)
    const int p = lp[y];
    if (p < r) lp[y] = r;
    y = p;
  }
  return r;
}

__device__ __forceinline__ void lunite(int* lp, int a, int b, int* err) {
  int ra = lfind(lp, a, err), rb = lfind(lp, b, err);
  int it = 0;
  while (ra != rb) {
    if (ra > rb) {
      const int t = ra;
      ra = rb;
      rb = t;
    }
    const int old = atomicCAS(&lp[ra], ra, rb);
    if (old == ra) return;
    ra = lfind(lp, old, err);
    rb = lfind(lp, rb, err);
    if (++it > 4 * kTileN) {
      *err |= ERR_UF_LIMIT;
      return;
    }
  }
}

// offsets of the 13 neighbours that precede a voxel in linear order
__device__ __forceinline__ void back_offset(int m, int& di, int& dj, int& dk) {
  if (m < 9) {
    dk = -1;
    dj = m / 3 - 1;
    di = m % 3 - 1;
  } else if (m < 12) {
    dk = 0;
    dj = -1;
    di = m - 10;
  } else {
    dk = 0;
    dj = 0;
    di = -1;
  }
}

// tile-local labelling; writes parent[] for every voxel of the tile
// (background 0, foreground the global index of its local root)
__global__ void __launch_bounds__(kTileThreads) k_uf_tile(Box b, const unsigned char* __restrict__ bin, int* parent,
                                                          Ctl* ctl) {
  __shared__ int lp[kTileN];
  __shared__ unsigned char lb[kTileN];
  const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile, z0 = blockIdx.z * kTile;
  int err = 0;
  for (int l = threadIdx.x; l < kTileN; l += kTileThreads) {
    const int li = l % kTile, lj = (l / kTile) % kTile, lk = l / (kTile * kTile);
    const int i = x0 + li, j = y0 + lj, k = z0 + lk;
    const bool in = i < b.nx && j < b.ny && k < b.nz;
    const unsigned char v = in ? bin[b.idx(i, j, k)] : 0;
    lb[l] = v;
    lp[l] = l;
  }
  __syncthreads();
  for (int l = threadIdx.x; l < kTileN; l += kTileThreads) {
    if (!lb[l]) continue;
    const int li = l % kTile, lj = (l / kTile) % kTile, lk = l / (kTile * kTile);
#pragma unroll
    for (int m = 0; m < 13; m++) {
      int di, dj, dk;
      back_offset(m, di, dj, dk);
      const int a = li + di, c = lj + dj, d = lk + dk;
      if (a < 0 || c < 0 || d < 0 || a >= kTile || c >= kTile) continue;
      const int l2 = a + kTile * (c + kTile * d);
      if (lb[l2]) lunite(lp, l, l2, &err);
    }
  }
  __syncthreads();
  for (int l = threadIdx.x; l < kTileN; l += kTileThreads) {
    const int li = l % kTile, lj = (l / kTile) % kTile, lk = l / (kTile * kTile);
    const int i = x0 + li, j = y0 + lj, k = z0 + lk;
    if (i >= b.nx || j >= b.ny || k >= b.nz) continue;
    int g = 0;
    if (lb[l]) {
      const int r = lfind(lp, l, &err);
      const int ri = r % kTile, rj = (r / kTile) % kTile, rk = r / (kTile * kTile);
      g = (int)b.idx(x0 + ri, y0 + rj, z0 + rk);
    }
    parent[b.idx(i, j, k)] = g;
  }
  if (err && ctl) atomicOr(&ctl->err, err);
}

// unions across tile faces: each voxel on a face of its tile with its
// preceding neighbours in other tiles.  Neighbouring voxels mostly join the
// same two tile components, so the lanes of a warp first agree on distinct
// (parent, parent) pairs and only one lane per pair unites them (the parents
// are in the same sets as the voxels).
// Preceding offsets have di, dj in {-1, 0, 1} and dk in {-1, 0}, so only the
// voxels of the tile's bottom plane (lk = 0) and of the ring li or lj in
// {0, kTile-1} of every other plane have one outside the tile: 64 + 7 x 28 =
// 260 of the 512.  face_voxel(f) enumerates them.
constexpr int kFaceN = kTile * kTile + (kTile - 1) * 4 * (kTile - 1);

__device__ __forceinline__ void face_voxel(int f, int& li, int& lj, int& lk) {
  if (f < kTile * kTile) {
    lk = 0;
    li = f % kTile;
    lj = f / kTile;
    return;
  }
  const int g = f - kTile * kTile, ring = 4 * (kTile - 1);
  lk = 1 + g / ring;
  const int r = g % ring;
  if (r < kTile) {
    lj = 0;
    li = r;
  } else if (r < 2 * kTile) {
    lj = kTile - 1;
    li = r - kTile;
  } else if (r < 3 * kTile - 2) {
    li = 0;
    lj = 1 + (r - 2 * kTile);
  } else {
    li = kTile - 1;
    lj = 1 + (r - (3 * kTile - 2));
  }
}

__global__ void __launch_bounds__(kTileThreads) k_uf_cross(Box b, const unsigned char* __restrict__ bin, int* parent,
                                                           Ctl* ctl) {
  const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile, z0 = blockIdx.z * kTile;
  const unsigned lane = threadIdx.x & 31u;
  int err = 0;
  // the tile's face voxels, one per thread (warp-uniform loop: a warp runs a
  // round while its first voxel exists)
  for (int base = threadIdx.x - (int)lane; base < kFaceN; base += kTileThreads) {
    const int l = base + (int)lane;
    int li = 0, lj = 0, lk = 0;
    if (l < kFaceN) face_voxel(l, li, lj, lk);
    const int i = x0 + li, j = y0 + lj, k = z0 + lk;
    const bool in = l < kFaceN && i < b.nx && j < b.ny && k < b.nz;
    const int64_t q = in ? b.idx(i, j, k) : 0;
    const bool fg = in && bin[q];
#pragma unroll 1
    for (int m = 0; m < 13; m++) {
      int di, dj, dk;
      back_offset(m, di, dj, dk);
      int ra = -1, rb = -1;
      if (fg) {
        const int a = li + di, c = lj + dj, d = lk + dk;
        const bool other_tile = !(a >= 0 && c >= 0 && d >= 0 && a < kTile && c < kTile);
        const int i2 = i + di, j2 = j + dj, k2 = k + dk;
        if (other_tile && i2 >= 0 && j2 >= 0 && k2 >= 0 && i2 < b.nx && j2 < b.ny) {
          const int64_t q2 = b.idx(i2, j2, k2);
          if (bin[q2]) {
            ra = __ldcg(parent + q);
            rb = __ldcg(parent + q2);
          }
        }
      }
      const bool pair = ra >= 0 && ra != rb;
      const unsigned lo = (unsigned)(ra < rb ? ra : rb), hi = (unsigned)(ra < rb ? rb : ra);
      const unsigned long long key =
          pair ? (((unsigned long long)lo << 32) | hi) : (0xffffffff00000000ull | lane);
      const unsigned peers = __match_any_sync(0xffffffffu, key);
      if (pair && (unsigned)(__ffs(peers) - 1) == lane) unite(parent, ra, rb, &err);
    }
  }
  if (err && ctl) atomicOr(&ctl->err, err);
}

__global__ void k_uf_final(int64_t n, const unsigned char* __restrict__ bin, int* parent, Ctl* ctl) {
  int err = 0;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    if (bin[q]) {
      int r = (int)q;
      int it = 0;
      while (parent[r] != r && it++ < kWalkCap) r = parent[r];
      if (it > kWalkCap) err |= ERR_UF_LIMIT;
      parent[q] = r;
    }
  }
  if (err && ctl) atomicOr(&ctl->err, err);
}

// MERGE_SETS(phi, mask_nw) then phi_bin = phi < 0 (trapComponents.c:167-170)
__global__ void k_bin_nw(int64_t n, double* phi, const double* __restrict__ mask_nw, unsigned char* bin) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double m = mask_nw[q];
    double p = phi[q];
    if (m > 0) {
      p = -m;
      phi[q] = p;
    }
    bin[q] = (p < 0.0) ? 1 : 0;
  }
}

// inlet / outlet reservoirs of trapComponents.c:175-194 and 257-299
__global__ void k_set_bin_slab(Box b, unsigned char* bin, int center, int outlet) {
  const int64_t nxy = (int64_t)b.nx * b.ny;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (!outlet) {
    if (center) {
      const int k = (int)(0.5 * (b.klo + b.khi)), i = (int)(0.5 * (b.ilo + b.ihi));
      if (t < b.ny) bin[i + (int64_t)t * b.nx + k * nxy] = 1;
    } else {
      const int i = b.ilo - 1;
      const int64_t cnt = (int64_t)b.fby() * b.fbz();
      if (t < cnt) {
        const int j = b.jlo + t % b.fby(), k = b.klo + t / b.fby();
        bin[i + (int64_t)j * b.nx + k * nxy] = 1;
      }
    }
  } else {
    if (center) {
      if (t < nxy) {
        bin[(int64_t)(b.klo - 1) * nxy + t] = 1;
        bin[(int64_t)(b.khi + 1) * nxy + t] = 1;
      }
      if (t < (int64_t)b.ny * b.nz) {
        const int j = t % b.ny, k = t / b.ny;
        bin[(b.ilo - 1) + (int64_t)j * b.nx + k * nxy] = 1;
        bin[(b.ihi + 1) + (int64_t)j * b.nx + k * nxy] = 1;
      }
    } else {
      const int i = b.ihi + 1;
      const int64_t cnt = (int64_t)b.fby() * b.fbz();
      if (t < cnt) {
        const int j = b.jlo + t % b.fby(), k = b.klo + t / b.fby();
        bin[i + (int64_t)j * b.nx + k * nxy] = 1;
      }
    }
  }
}

// trapComponents.c:226-259: disconnected non-wetting mask, then the masked
// wetting phase in scratch and its binary image
__global__ void k_trap_nw(int64_t n, const int* __restrict__ labels, int main_idx, const double* __restrict__ phi,
                          const double* __restrict__ mask, double* mask_nw, double* scratch, unsigned char* bin,
                          double fill) {
  const int main_label = labels[main_idx];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int l = labels[q];
    const bool disc = !(l == main_label || l == 0);
    const double p = phi[q];
    const double mnw = (disc && p < 0) ? -p : fill;
    mask_nw[q] = mnw;
    double s = -p;
    const double m = mask[q];
    s = (m > s) ? m : s;
    s = (mnw > s) ? mnw : s;
    scratch[q] = s;
    bin[q] = (s < 0.0) ? 1 : 0;
  }
}

__global__ void k_trap_w(int64_t n, const int* __restrict__ labels, int main_idx, const double* __restrict__ scratch,
                         double* mask_w, double fill) {
  const int main_label = labels[main_idx];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int l = labels[q];
    const bool disc = !(l == main_label || l == 0);
    const double s = scratch[q];
    mask_w[q] = (disc && s < 0) ? -s : fill;
  }
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

void launch_label(cudaStream_t s, const Box& b, const unsigned char* bin, int* labels, Ctl* ctl) {
  const int64_t n = b.npts();
  const dim3 tiles((b.nx + kTile - 1) / kTile, (b.ny + kTile - 1) / kTile, (b.nz + kTile - 1) / kTile);
  k_uf_tile<<<tiles, kTileThreads, 0, s>>>(b, bin, labels, ctl);
  k_uf_cross<<<tiles, kTileThreads, 0, s>>>(b, bin, labels, ctl);
  k_uf_final<<<grid_for(n), 256, 0, s>>>(n, bin, labels, ctl);
}

void launch_bin_nw(cudaStream_t s, int64_t n, double* phi, const double* mask_nw, unsigned char* bin) {
  k_bin_nw<<<grid_for(n), 256, 0, s>>>(n, phi, mask_nw, bin);
}

void launch_set_bin_slab(cudaStream_t s, const Box& b, unsigned char* bin, int center_inlet, int outlet) {
  int64_t cnt = (int64_t)b.nx * b.ny;
  if ((int64_t)b.ny * b.nz > cnt) cnt = (int64_t)b.ny * b.nz;
  if ((int64_t)b.fby() * b.fbz() > cnt) cnt = (int64_t)b.fby() * b.fbz();
  k_set_bin_slab<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(b, bin, center_inlet, outlet);
}

void launch_trap_nw(cudaStream_t s, int64_t n, const int* labels, int main_idx, const double* phi,
                    const double* mask, double* mask_nw, double* scratch, unsigned char* bin, double fill) {
  k_trap_nw<<<grid_for(n), 256, 0, s>>>(n, labels, main_idx, phi, mask, mask_nw, scratch, bin, fill);
}

void launch_trap_w(cudaStream_t s, int64_t n, const int* labels, int main_idx, const double* scratch,
                   double* mask_w, double fill) {
  k_trap_w<<<grid_for(n), 256, 0, s>>>(n, labels, main_idx, scratch, mask_w, fill);
}

}  // namespace qss
