// Placement of a newly added system on the device: particles uploaded in input
// order into the rebin scratch (t_*) are put in cell order, in input order
// within each cell, exactly as the host bucketing of xnb_system_add does
// (domain_periodic_location, core/include/exanb/core/domain.h:160-191, with the
// wrap of positions by whole cells).
#include "xnb_launch.cuh"

namespace xnb {

namespace {

// cell of each particle, wrapped position, and an arrival slot in its cell (unordered)
__global__ void __launch_bounds__(256) k_place_cell(PlaceArgs P, DevArrays a, unsigned int* flags) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < P.n; q += gridDim.x * blockDim.x) {
    const uint32_t i = P.poff + q;
    double r[3] = {a.t_rx[i], a.t_ry[i], a.t_rz[i]};
    int loc[3];
    bool bad = false;
    for (int ax = 0; ax < 3; ++ax) {
      const double rel = __dsub_rn(r[ax], P.origin[ax]);
      const double qd = floor(__ddiv_rn(rel, P.cell_size));
      if (!(fabs(qd) < 1.0e9)) {
        bad = true;
        loc[ax] = 0;
        continue;
      }
      long long l = static_cast<long long>(qd);
      if (l < 0 || l >= P.dims[ax]) {
        const long long old = l;
        l = ((l % P.dims[ax]) + P.dims[ax]) % P.dims[ax];
        r[ax] = __dadd_rn(r[ax], __dmul_rn(static_cast<double>(l - old), P.cell_size));
      }
      loc[ax] = static_cast<int>(l);
    }
    if (bad) atomicOr(flags, 1u);
    a.t_rx[i] = r[0];
    a.t_ry[i] = r[1];
    a.t_rz[i] = r[2];
    const uint32_t c = static_cast<uint32_t>((loc[2] * P.dims[1] + loc[1]) * P.dims[0] + loc[0]);
    a.pdest[i] = c;
    a.plocal[i] = atomicAdd(&a.cell_cnt[P.coff + c], 1u);
  }
}

// input indices grouped by cell (unordered inside a cell)
__global__ void __launch_bounds__(256)
    k_place_slots(PlaceArgs P, DevArrays a, const unsigned long long* __restrict__ start) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < P.n; q += gridDim.x * blockDim.x) {
    const uint32_t i = P.poff + q;
    a.mover_list[P.poff + static_cast<uint32_t>(start[a.pdest[i]]) + a.plocal[i]] = q;
  }
}

// One warp per cell: a member's place is the number of members with a smaller
// input index (input order kept), then its data moves into place.
__global__ void __launch_bounds__(128)
    k_place_order(PlaceArgs P, DevArrays a, const unsigned long long* __restrict__ start, unsigned int* flags) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < P.ncells; c += warps) {
    const uint32_t s0 = static_cast<uint32_t>(start[c]);
    const uint32_t nc = static_cast<uint32_t>(start[c + 1]) - s0;
    const uint32_t* members = a.mover_list + P.poff + s0;
    if (nc > kPlaceMaxCell) {
      if (lane == 0) atomicOr(flags, 2u);  // the host places this system instead
      continue;
    }
    for (uint32_t k = lane; k < nc; k += 32) {
      const uint32_t qk = members[k];
      uint32_t rank = 0;
      for (uint32_t m = 0; m < nc; ++m) rank += members[m] < qk ? 1u : 0u;
      const uint32_t src = P.poff + qk, dst = P.poff + s0 + rank;
      const double x = a.t_rx[src], y = a.t_ry[src], z = a.t_rz[src];
      a.rx[dst] = x;
      a.ry[dst] = y;
      a.rz[dst] = z;
      a.vx[dst] = a.t_vx[src];
      a.vy[dst] = a.t_vy[src];
      a.vz[dst] = a.t_vz[src];
      a.id[dst] = a.t_id[src];
      a.ptype[dst] = 0;
      a.pcell[dst] = P.coff + c;
      const double ox = x - P.origin[0], oy = y - P.origin[1], oz = z - P.origin[2];
      const float4 hi = make_float4(static_cast<float>(ox), static_cast<float>(oy), static_cast<float>(oz), 0.f);
      a.pf[dst] = hi;
      a.pflo[dst] = make_float4(static_cast<float>(ox - static_cast<double>(hi.x)),
                                static_cast<float>(oy - static_cast<double>(hi.y)),
                                static_cast<float>(oz - static_cast<double>(hi.z)), 0.f);
      a.fx[dst] = 0.0;
      a.fy[dst] = 0.0;
      a.fz[dst] = 0.0;
      a.pe[dst] = 0.0;
      a.nbr_cnt[dst] = 0;
      a.nbr_start[dst] = 0;
    }
    if (lane == 0) {
      a.cell_start[P.coff + c] = P.poff + s0;
      a.cell_n[P.coff + c] = nc;
      a.cell_sys[P.coff + c] = P.sys_slot;
    }
  }
}

}  // namespace

int launch_place(const PlaceArgs& P, const DevArrays& a, unsigned int* flags, int sm_count, cudaStream_t stream) {
  if (P.n == 0 || P.ncells == 0) return 0;
  int count = 0;
  const long long tb = (static_cast<long long>(P.n) + 255) / 256;
  const int gt = static_cast<int>(tb > sm_count * 16LL ? sm_count * 16LL : tb);
  cudaMemsetAsync(a.cell_cnt + P.coff, 0, static_cast<size_t>(P.ncells) * sizeof(uint32_t), stream);
  k_place_cell<<<gt, 256, 0, stream>>>(P, a, flags);
  ++count;
  unsigned long long* start = a.cell_scan + P.coff;
  count += launch_scan_u32_to_u64(a.cell_cnt + P.coff, start, P.ncells, a.scan_blocks, stream);
  k_place_slots<<<gt, 256, 0, stream>>>(P, a, start);
  ++count;
  const long long wb = (static_cast<long long>(P.ncells) + 3) / 4;
  const int gw = static_cast<int>(wb > sm_count * 16LL ? sm_count * 16LL : wb);
  k_place_order<<<gw, 128, 0, stream>>>(P, a, start, flags);
  ++count;
  return count;
}

}  // namespace xnb
