// Multi-rank halo: host-side index maps that split one sparse-block geometry over
// ranks, in the terms of this library's block layout.
//
// The reference splits its domain with ParMETIS and exchanges, once per step, the
// distributions each rank streams into sites another rank owns
// (geometry::FieldData::SendAndReceive / CopyReceived, Code/geometry/FieldData.cc:
// 27-49), streaming the sites that have off-rank neighbours first and the others
// while the exchange is in flight (Code/lb/lb.hpp:176-309).  Here:
//
// * Partition (hlbg_halo_partition): contiguous ranges of the device block order
//   (z-columns: 2-D Morton order of the block's (x, y), then z), cut where the
//   running fluid-site count passes k*N/R, so ranks get equal site counts and
//   mostly whole z-columns.
// * Local geometry (hlbg_halo_create): the rank's owned blocks, then as ghost
//   blocks every block of another rank among the 26 neighbours of an owned block,
//   with the link records of all their sites; every owned site therefore sees its
//   whole neighbourhood exactly as in the global geometry.
// * Exchange lists: for each peer, the distributions this rank streams into the
//   peer's sites (send) and the ones the peer streams into this rank's sites
//   (receive), as (local block, direction, in-block site) triples.  Both sides list
//   one exchange in the same order -- ascending (input block, site, direction) of
//   the target -- so the receiver scatters the sender's buffer element by element.
// * Edge blocks: owned blocks with a site that streams into a ghost block.  They
//   must be updated before the send; the other owned blocks can be updated while
//   the exchange runs.  The receive writes only target slots no owned site
//   streams into, and it must complete before PostStep (the BFL PostStep reads
//   a site's own new distributions, some of which arrive from peers).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/hemelb_gb300.h"

namespace {

const int HCX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int HCY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int HCZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};

// The device layout's default block order (z-columns, capi.cu build_layout).
uint64_t zcolumn_key(uint32_t x, uint32_t y, uint32_t z) {
  uint64_t m = 0;
  for (int k = 0; k < 16; ++k) {
    m |= (uint64_t)((x >> k) & 1u) << (3 * k + 2);
    m |= (uint64_t)((y >> k) & 1u) << (3 * k + 1);
  }
  return (m << 16) | (uint64_t)z;
}

int popcount64(uint64_t v) {
  int c = 0;
  while (v) {
    v &= v - 1;
    ++c;
  }
  return c;
}

struct Peer {
  int32_t rank = -1;
  std::vector<int32_t> send_block, recv_block;
  std::vector<int8_t> send_dir, recv_dir;
  std::vector<int16_t> send_site, recv_site;
};

// Validated view of the input geometry with a block-grid lookup.
struct Input {
  const hlbg_geometry* g = nullptr;
  int64_t nb = 0;
  int NX = 0, NY = 0, NZ = 0;
  std::vector<int32_t> grid;  // block grid -> input block index, -1 empty
  int check(std::string* err) {
    nb = g->n_blocks;
    NX = g->blocks[0];
    NY = g->blocks[1];
    NZ = g->blocks[2];
    if (g->q != 19 && g->q != 15) return *err = "q must be 19 or 15", HLBG_ERR_INVAL;
    if (g->block_size != 8) return *err = "block_size must be 8", HLBG_ERR_INVAL;
    if (nb <= 0 || !g->block_coords || !g->fluid_mask || NX <= 0 || NY <= 0 || NZ <= 0)
      return *err = "geometry has no blocks", HLBG_ERR_INVAL;
    if ((int64_t)NX * NY * NZ > (1ll << 31) || nb >= (1ll << 31) / 512)
      return *err = "block grid too large", HLBG_ERR_INVAL;
    grid.assign((size_t)NX * NY * NZ, -1);
    for (int64_t b = 0; b < nb; ++b) {
      const int32_t x = g->block_coords[3 * b], y = g->block_coords[3 * b + 1], z = g->block_coords[3 * b + 2];
      if (x < 0 || y < 0 || z < 0 || x >= NX || y >= NY || z >= NZ)
        return *err = "block coordinate outside the block grid", HLBG_ERR_INVAL;
      int32_t& cell = grid[((size_t)x * NY + y) * NZ + z];
      if (cell >= 0) return *err = "duplicate block coordinates", HLBG_ERR_INVAL;
      cell = (int32_t)b;
    }
    if (g->n_link_sites < 0 || (g->n_link_sites && (!g->link_site || !g->wall_mask || !g->iolet_mask ||
                                                    !g->iolet_id || !g->site_type)))
      return *err = "bad link-site arrays", HLBG_ERR_INVAL;
    for (int64_t r = 0; r < g->n_link_sites; ++r)
      if (g->link_site[r] < 0 || g->link_site[r] >= nb * 512 || (r && g->link_site[r] <= g->link_site[r - 1]))
        return *err = "link sites must be ascending and inside the blocks", HLBG_ERR_INVAL;
    return HLBG_OK;
  }
  bool fluid(int64_t b, int l) const { return (g->fluid_mask[b * 8 + (l >> 6)] >> (l & 63)) & 1ull; }
  int32_t block_at(int x, int y, int z) const {
    if (x < 0 || y < 0 || z < 0 || x >= NX || y >= NY || z >= NZ) return -1;
    return grid[((size_t)x * NY + y) * NZ + z];
  }
  // neighbour of site (b, l) along direction d: (block, local site), block -1 if none
  std::pair<int32_t, int> neighbour(int64_t b, int l, int d) const {
    const int x = (l >> 6) + HCX[d], y = ((l >> 3) & 7) + HCY[d], z = (l & 7) + HCZ[d];
    const int32_t* c = g->block_coords + 3 * b;
    const int32_t nbk = block_at(c[0] + (x >> 3), c[1] + (y >> 3), c[2] + (z >> 3));
    return {nbk, ((x & 7) * 8 + (y & 7)) * 8 + (z & 7)};
  }
  // link record of site (b, l), -1 without one (link_site is ascending)
  int64_t record(int64_t b, int l) const {
    const int64_t key = b * 512 + l;
    const int64_t* p = std::lower_bound(g->link_site, g->link_site + g->n_link_sites, key);
    return (p != g->link_site + g->n_link_sites && *p == key) ? (int64_t)(p - g->link_site) : -1;
  }
  // does site (b, l) stream along d into its neighbour?  Not when the link is a wall
  // or iolet link (StreamerTypeFactory: iolet, then wall, then bulk), nor when the
  // neighbour is not a fluid site (the reference's rubbish slot).
  bool streams(int64_t b, int l, int d, int32_t* nb_out, int* nl_out) const {
    const int64_t r = record(b, l);
    if (r >= 0 && ((g->wall_mask[r] | g->iolet_mask[r]) >> (d - 1)) & 1u) return false;
    auto [nbk, nl] = neighbour(b, l, d);
    if (nbk < 0 || !fluid(nbk, nl)) return false;
    *nb_out = nbk;
    *nl_out = nl;
    return true;
  }
};

}  // namespace

struct hlbg_halo {
  std::string err;
  int32_t rank = 0, n_ranks = 1;
  int q = 19;
  int grid[3] = {0, 0, 0};
  int64_t n_owned = 0;
  std::vector<int64_t> source;  // local block -> input block
  std::vector<int32_t> block_coords;
  std::vector<uint64_t> fluid_mask;
  std::vector<int64_t> link_site;
  std::vector<uint32_t> wall_mask, iolet_mask;
  std::vector<int32_t> iolet_id;
  std::vector<int8_t> site_type;
  std::vector<float> cuts, normals;
  bool has_cuts = false, has_normals = false;
  std::vector<uint8_t> edge;  // per owned block
  std::vector<Peer> peers;
};

extern "C" {

int hlbg_halo_partition(const hlbg_geometry* g, int32_t n_ranks, int32_t* block_rank) {
  if (!g || !block_rank || n_ranks < 1) return HLBG_ERR_INVAL;
  Input in;
  in.g = g;
  std::string err;
  int rc = in.check(&err);
  if (rc) return rc;
  std::vector<std::pair<uint64_t, int64_t>> order((size_t)in.nb);
  int64_t total = 0;
  for (int64_t b = 0; b < in.nb; ++b) {
    const int32_t* c = g->block_coords + 3 * b;
    order[b] = {zcolumn_key((uint32_t)c[0], (uint32_t)c[1], (uint32_t)c[2]), b};
    for (int w = 0; w < 8; ++w) total += popcount64(g->fluid_mask[b * 8 + w]);
  }
  std::sort(order.begin(), order.end());
  int64_t before = 0;
  for (const auto& [key, b] : order) {
    (void)key;
    // the rank whose share [k N/R, (k+1) N/R) holds this block's first site
    int64_t r = total ? (before * n_ranks) / total : 0;
    block_rank[b] = (int32_t)std::min<int64_t>(r, n_ranks - 1);
    for (int w = 0; w < 8; ++w) before += popcount64(g->fluid_mask[b * 8 + w]);
  }
  return HLBG_OK;
}

int hlbg_halo_create(const hlbg_geometry* g, const int32_t* block_rank, int32_t n_ranks, int32_t rank,
                     hlbg_halo** out) {
  if (!out) return HLBG_ERR_INVAL;
  *out = nullptr;
  if (!g || !block_rank || n_ranks < 1 || rank < 0 || rank >= n_ranks) return HLBG_ERR_INVAL;
  hlbg_halo* h = new (std::nothrow) hlbg_halo();
  if (!h) return HLBG_ERR_OOM;
  *out = h;  // returned on failure too, for hlbg_halo_last_error; the caller destroys it
  Input in;
  in.g = g;
  int rc = in.check(&h->err);
  if (rc) return rc;
  if (g->q != 19) return h->err = "exchange lists are built for D3Q19", HLBG_ERR_INVAL;
  for (int64_t b = 0; b < in.nb; ++b)
    if (block_rank[b] < 0 || block_rank[b] >= n_ranks) return h->err = "block rank out of range", HLBG_ERR_INVAL;
  h->rank = rank;
  h->n_ranks = n_ranks;
  h->q = g->q;
  for (int a = 0; a < 3; ++a) h->grid[a] = g->blocks[a];
  auto key_of = [&](int64_t b) {
    const int32_t* c = g->block_coords + 3 * b;
    return zcolumn_key((uint32_t)c[0], (uint32_t)c[1], (uint32_t)c[2]);
  };
  // owned blocks, then ghost blocks (26-neighbours of owned blocks on other ranks)
  std::vector<std::pair<uint64_t, int64_t>> owned, ghost;
  std::vector<uint8_t> is_ghost((size_t)in.nb, 0);
  for (int64_t b = 0; b < in.nb; ++b) {
    if (block_rank[b] != rank) continue;
    owned.push_back({key_of(b), b});
    const int32_t* c = g->block_coords + 3 * b;
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          const int32_t nb = in.block_at(c[0] + dx, c[1] + dy, c[2] + dz);
          if (nb >= 0 && block_rank[nb] != rank && !is_ghost[nb]) {
            is_ghost[nb] = 1;
            ghost.push_back({key_of(nb), nb});
          }
        }
  }
  std::sort(owned.begin(), owned.end());
  std::sort(ghost.begin(), ghost.end());
  h->n_owned = (int64_t)owned.size();
  std::vector<int32_t> local_of((size_t)in.nb, -1);
  for (const auto* list : {&owned, &ghost})
    for (const auto& kb : *list) {
      local_of[kb.second] = (int32_t)h->source.size();
      h->source.push_back(kb.second);
    }
  // local geometry: blocks, fluid masks and the link records of all their sites
  const int64_t nl = (int64_t)h->source.size();
  const int nq = g->q - 1;
  h->has_cuts = g->cut_distance != nullptr;
  h->has_normals = g->wall_normal != nullptr;
  for (int64_t lb = 0; lb < nl; ++lb) {
    const int64_t b = h->source[lb];
    for (int a = 0; a < 3; ++a) h->block_coords.push_back(g->block_coords[3 * b + a]);
    for (int w = 0; w < 8; ++w) h->fluid_mask.push_back(g->fluid_mask[b * 8 + w]);
    const int64_t* lo = std::lower_bound(g->link_site, g->link_site + g->n_link_sites, b * 512);
    const int64_t* hi = std::lower_bound(lo, g->link_site + g->n_link_sites, (b + 1) * 512);
    for (const int64_t* p = lo; p < hi; ++p) {
      const int64_t r = p - g->link_site;
      h->link_site.push_back(lb * 512 + (*p - b * 512));
      h->wall_mask.push_back(g->wall_mask[r]);
      h->iolet_mask.push_back(g->iolet_mask[r]);
      h->iolet_id.push_back(g->iolet_id[r]);
      h->site_type.push_back(g->site_type[r]);
      if (h->has_cuts) h->cuts.insert(h->cuts.end(), g->cut_distance + r * nq, g->cut_distance + (r + 1) * nq);
      if (h->has_normals) h->normals.insert(h->normals.end(), g->wall_normal + 3 * r, g->wall_normal + 3 * r + 3);
    }
  }
  // exchange lists, keyed (target input block, target site, direction)
  using Key = std::tuple<int64_t, int, int>;
  std::vector<std::vector<Key>> send((size_t)n_ranks), recv((size_t)n_ranks);
  h->edge.assign((size_t)h->n_owned, 0);
  for (int64_t lb = 0; lb < h->n_owned; ++lb) {
    const int64_t b = h->source[lb];
    for (int l = 0; l < 512; ++l) {
      if (!in.fluid(b, l)) continue;
      for (int d = 1; d < 19; ++d) {
        int32_t tb;
        int tl;
        // this site streams into a peer's site: send
        if (in.streams(b, l, d, &tb, &tl) && block_rank[tb] != rank) {
          send[block_rank[tb]].push_back({tb, tl, d});
          h->edge[lb] = 1;
        }
        // a peer's site streams into this one along d: receive.  Its upstream site
        // is the neighbour against d, i.e. along the opposite direction.
        const int x = (l >> 6) - HCX[d], y = ((l >> 3) & 7) - HCY[d], z = (l & 7) - HCZ[d];
        const int32_t* c = g->block_coords + 3 * b;
        const int32_t ub = in.block_at(c[0] + (x >> 3), c[1] + (y >> 3), c[2] + (z >> 3));
        if (ub < 0 || block_rank[ub] == rank) continue;
        const int ul = ((x & 7) * 8 + (y & 7)) * 8 + (z & 7);
        if (in.fluid(ub, ul) && in.streams(ub, ul, d, &tb, &tl)) recv[block_rank[ub]].push_back({b, l, d});
      }
    }
  }
  for (int32_t p = 0; p < n_ranks; ++p) {
    if (send[p].empty() && recv[p].empty()) continue;
    std::sort(send[p].begin(), send[p].end());
    std::sort(recv[p].begin(), recv[p].end());
    Peer pr;
    pr.rank = p;
    for (const auto& [tb, tl, d] : send[p]) {
      pr.send_block.push_back(local_of[tb]);
      pr.send_site.push_back((int16_t)tl);
      pr.send_dir.push_back((int8_t)d);
    }
    for (const auto& [tb, tl, d] : recv[p]) {
      pr.recv_block.push_back(local_of[tb]);
      pr.recv_site.push_back((int16_t)tl);
      pr.recv_dir.push_back((int8_t)d);
    }
    h->peers.push_back(std::move(pr));
  }
  return HLBG_OK;
}

void hlbg_halo_destroy(hlbg_halo* h) { delete h; }

const char* hlbg_halo_last_error(const hlbg_halo* h) { return h ? h->err.c_str() : "null halo"; }

int hlbg_halo_local_geometry(const hlbg_halo* h, hlbg_geometry* out, int64_t* n_owned_blocks) {
  if (!h || !out) return HLBG_ERR_INVAL;
  std::memset(out, 0, sizeof(*out));
  out->q = h->q;
  out->block_size = 8;
  for (int a = 0; a < 3; ++a) out->blocks[a] = h->grid[a];
  out->n_blocks = (int64_t)h->source.size();
  out->block_coords = h->block_coords.data();
  out->fluid_mask = h->fluid_mask.data();
  out->n_link_sites = (int64_t)h->link_site.size();
  out->link_site = h->link_site.data();
  out->wall_mask = h->wall_mask.data();
  out->iolet_mask = h->iolet_mask.data();
  out->iolet_id = h->iolet_id.data();
  out->site_type = h->site_type.data();
  out->cut_distance = h->has_cuts ? h->cuts.data() : nullptr;
  out->wall_normal = h->has_normals ? h->normals.data() : nullptr;
  if (n_owned_blocks) *n_owned_blocks = h->n_owned;
  return HLBG_OK;
}

int hlbg_halo_block_source(const hlbg_halo* h, int64_t* input_block) {
  if (!h || !input_block) return HLBG_ERR_INVAL;
  std::copy(h->source.begin(), h->source.end(), input_block);
  return HLBG_OK;
}

int hlbg_halo_edge_blocks(const hlbg_halo* h, uint8_t* is_edge) {
  if (!h || !is_edge) return HLBG_ERR_INVAL;
  std::copy(h->edge.begin(), h->edge.end(), is_edge);
  return HLBG_OK;
}

int32_t hlbg_halo_peer_count(const hlbg_halo* h) { return h ? (int32_t)h->peers.size() : -1; }

int hlbg_halo_peer(const hlbg_halo* h, int32_t k, int32_t* peer_rank, int64_t* n_send, int64_t* n_recv) {
  if (!h || k < 0 || k >= (int32_t)h->peers.size()) return HLBG_ERR_INVAL;
  const Peer& p = h->peers[k];
  if (peer_rank) *peer_rank = p.rank;
  if (n_send) *n_send = (int64_t)p.send_block.size();
  if (n_recv) *n_recv = (int64_t)p.recv_block.size();
  return HLBG_OK;
}

int hlbg_halo_list(const hlbg_halo* h, int32_t k, int32_t is_recv, int32_t* local_block, int8_t* direction,
                   int16_t* site) {
  if (!h || k < 0 || k >= (int32_t)h->peers.size() || !local_block || !direction || !site)
    return HLBG_ERR_INVAL;
  const Peer& p = h->peers[k];
  const auto& b = is_recv ? p.recv_block : p.send_block;
  const auto& d = is_recv ? p.recv_dir : p.send_dir;
  const auto& s = is_recv ? p.recv_site : p.send_site;
  std::copy(b.begin(), b.end(), local_block);
  std::copy(d.begin(), d.end(), direction);
  std::copy(s.begin(), s.end(), site);
  return HLBG_OK;
}

}  // extern "C"
