// Staged pair form: the host entry points, and the launches for P = 512 and
// 1024 (staged_core.cuh holds the kernel; pairs_staged_large.cu launches
// P = 2048 and 4096).
#include "staged_core.cuh"

namespace seismic {

// The staged form serves P = 512 .. 4096: there the three rows of a couple
// (3 x C x 4P bytes) outgrow what L1 keeps and the direct form waits on L2
// (measured, staged vs direct M pairs/s: P=512 C=1 973 vs 926, P=1024 C=1
// 549 vs 496, C=3 379 vs 339).  SEISMIC_PAIR_KERNEL=direct forces the direct
// form everywhere.
bool staged_enabled() { return !staged_disabled() && tensor_map_encoder() != nullptr; }

bool staged_supported(int P, const PairArgs &a) {
  if (P < 512 || P > 4096 || staged_disabled()) return false;
  if (a.stype < 0 || a.stype > 2) return false;
  if ((reinterpret_cast<uintptr_t>(a.spectra) & 15u) != 0) return false;
  if (a.rect && (reinterpret_cast<uintptr_t>(a.spectra_q) & 15u) != 0) return false;
  if (a.spectra_i && (reinterpret_cast<uintptr_t>(a.spectra_i) & 15u) != 0) return false;
  return tensor_map_encoder() != nullptr;
}

static StagedGeom staged_geom_of(int P, const PairArgs &a) {
  const int ng = staged_shape(P, a).nwarp * 32 / (P / 32);
  return staged_geom(ng, staged_item_rows(ng, a));
}

void staged_tiling(int P, const PairArgs &a, long long *tile_side, long long *items_per_tile) {
  const StagedGeom gm = staged_geom_of(P, a);
  *tile_side = gm.ts;
  *items_per_tile = gm.ipt;
}

long long staged_items_total(int P, const PairArgs &a) {
  const StagedGeom gm = staged_geom_of(P, a);
  if (a.rect) return (a.n_query + gm.ti - 1) / gm.ti * ((a.n_cols + gm.tj - 1) / gm.tj);
  const long long nb = (a.n_events + gm.ts - 1) / gm.ts;
  return gm.ipt * (nb * (nb + 1) / 2);
}

cudaError_t launch_pairs_staged_large(int P, const PairArgs &a, int sm_count, cudaStream_t s);

cudaError_t launch_pairs_staged(int P, const PairArgs &a, int sm_count, cudaStream_t s) {
  switch (P) {
    case 512: return launch_staged_p<512>(a, sm_count, s);
    case 1024: return launch_staged_p<1024>(a, sm_count, s);
    case 2048:
    case 4096: return launch_pairs_staged_large(P, a, sm_count, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
