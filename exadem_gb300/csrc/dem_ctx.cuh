// dem_ctx.cuh -- the library context (one simulated system) and the kernel
// launchers shared by the translation units of the GB300 DEM hot path.
#pragma once
#include <string>
#include <vector>

#include "dem_internal.cuh"

// Kernel classes for the built-in profiler (dem_profile / dem_kernel_stats).
enum DemKClass : int {
  K_PROLOG, K_DISPL, K_BIN, K_REORDER, K_BROAD_COUNT, K_BROAD_FILL, K_REVERSE, K_SCAN,
  K_CONTACT, K_GATHER, K_RESET, K_GRAVITY, K_F2A, K_EPILOG, K_STATE, K_CSCREEN, K_CDETECT, K_BOND, K_NCLASS
};
static const char* const kDemKClassNames[K_NCLASS] = {
    "prolog", "displ_over", "bin_cells", "reorder", "broad_count", "broad_fill", "reverse_lists", "scan",
    "contact", "gather", "reset", "gravity", "force_to_accel", "epilog", "state", "contact_screen",
    "contact_detect", "bonds"};

namespace dem {
struct MlpState;  // k_mlp.cu
}

// device scalars (d_scalars, u64): [0] rebuild trigger, [1] active contacts,
// [3..4] compaction list counts, [8] learned-record overflows, [12] interfaces broken,
// [16..23] learned bin counters and cursors (14 u32)
constexpr int DEM_NSCALARS = 32;
constexpr int SC_ROT_CNT = 6, SC_LEARNED_OVF = 8, SC_BROKEN = 12, SC_LEARNED_BINS = 16;

// features recorded per polyhedron unit by the count pass of the FP32-decided
// enumeration; the fill pass copies them instead of deciding again
constexpr int FEAT_SLOTS = 16;

// one mesh driver (dem_register_mesh): device arrays, the host copy of the
// world vertices and topology the bin grid is built from, and the sphere
// radius bound and skin the current bins were built for
struct MeshStore {
  double* vtx = nullptr;  // 3 nv: x | y | z
  int* e = nullptr;
  int* fo = nullptr;
  int* fv = nullptr;
  uint32_t* boff = nullptr;
  uint32_t* bitem = nullptr;
  float4* fsph = nullptr;
  std::vector<double> hx, hy, hz;
  std::vector<int> he, hfo, hfv;
  double bin_rad = -1.0, bin_skin = -1.0;
  dem::MeshDev dev{};
};

struct dem_ctx {
  dem_params prm{};
  cudaStream_t stream = nullptr;
  int device = 0;
  int num_sms = 152;
  std::string last_err;

  // particles (double-buffered for the cell reorder)
  uint64_t n = 0, pcap = 0;
  dem::PArrays P[2]{};
  void* pblock[2] = {nullptr, nullptr};
  int pcur = 0;
  double rad_max = 0.0;

  // drivers
  int ndrv = 0;
  dem::DriverDev drv_host[DEM_MAX_DRIVERS]{};
  dem::DriverDev* drv_dev = nullptr;
  std::vector<MeshStore> meshes;        // mesh drivers (DriverDev::mesh indexes)
  dem::MeshDev* mesh_dev = nullptr;     // device copy of meshes[k].dev
  uint32_t* mesh_cnt = nullptr;         // per sphere: mesh candidates of the last count pass
  uint64_t mesh_cnt_cap = 0;

  // systems (batched context); one system spanning prm's domain otherwise
  std::vector<dem_system> systems;   // empty: single system from prm
  int nsys = 1;
  dem::GridDev* grids_dev = nullptr;  // nsys each
  uint32_t* coff_dev = nullptr;       // nsys + 1
  uint64_t* pfirst_dev = nullptr;     // nsys + 1
  int2* drange_dev = nullptr;         // nsys
  uint32_t* trig_dev = nullptr;       // nsys: own trigger fired since the last rebuild
  int sys_cap = 0;
  dem::SysView sysview() const { return dem::SysView{grids_dev, coff_dev, pfirst_dev, drange_dev, trig_dev, nsys}; }

  // learned part (k_mlp.cu): MLP weights and training scratch
  dem::MlpState* mlp = nullptr;

  // launch shapes chosen by dem_autotune (no effect on results)
  int tune_block = 128;      // threads per block of the fused prolog / epilog (64..256)
  int tune_contact_bps = 8;  // persistent blocks per SM of the compacted contact law
  bool fuse_contact = true;  // compacted contact: detection and law in one kernel (k_cfused), else two
  int mul_mode = 2;          // multiply placement of the fused integration kernels (integrate_core.cuh)
  int tune_int_share = 0;    // k_cfused: Hooke tiles out of 8 whose arithmetic runs on the integer pipe
  int cell_broad_phase = 0;  // spheres, FP32 broad phase: warp per cell with staged neighbourhoods

  // graph step (dem_graph.cu)
  bool capturing = false;                  // kernels launched now go into a graph
  unsigned long long* d_gs = nullptr;      // [0] ni, [1] overflow, [2] rebuilds, [3] capacity
  unsigned long long* d_ni = nullptr;      // = d_gs
  uint64_t gcap = 0;                       // interaction capacity the graph was captured with
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool capturing_body = false;             // capturing the conditional rebuild
  uint64_t graph_launches_per_step[K_NCLASS] = {};     // kernel launches of one replay, per class
  uint64_t graph_launches_per_rebuild[K_NCLASS] = {};  // and of the conditional rebuild
  uint64_t gen = 0;        // bumped by every host-side change a captured graph depends on
  uint64_t graph_gen = ~0ull;
  void* snap = nullptr;                    // state snapshot for the overflow rollback
  uint64_t snap_bytes = 0;

  // cell grid (grid = system 0's, used by the single-system polyhedron path)
  dem::GridDev grid{};
  uint64_t ncell = 0, ccap = 0;
  uint32_t* cell_cnt = nullptr;    // ncell+1 (counts, then cursor)
  uint32_t* cell_start = nullptr;  // ncell+1
  uint32_t* cell_of = nullptr;     // n, cell of each particle (new order after reorder)
  uint32_t* cell_tmp = nullptr;    // n, cell of each particle in the old order
  uint32_t* perm = nullptr;        // n, new slot -> old slot
  uint32_t* pcnt = nullptr;        // n+1 candidate counts (then offsets)
  uint32_t* srec = nullptr;        // spheres: 8 (partner, meta) candidates per particle from the count pass
  float* crel[4] = {};             // n each: cell-relative x, y, z and radius in FP32 (broad phase)

  // interactions (double-buffered for the history carry-over)
  uint64_t ni = 0;
  uint64_t icap[2] = {0, 0};
  dem::IArrays I[2]{};
  uint32_t* own_off[2] = {nullptr, nullptr};  // n+1 each
  int icur = 0;
  bool have_list = false;   // list valid for the current particle state
  bool hist_valid = false;  // I[icur]/own_off[icur] usable as history for the next build
  uint64_t rcap = 0;
  dem::Records R{};
  uint32_t* rev_off = nullptr;  // n+1
  uint32_t* rev_cnt = nullptr;  // n+1
  unsigned int* rev_nlong = nullptr;  // reverse lists too long for a thread (k_rev_short -> k_rev_rank)
  uint32_t* rev_idx = nullptr;  // rcap
  // compacted contact passes (rcap each): work lists and detection results
  uint32_t* L1 = nullptr;
  uint32_t* L2 = nullptr;
  uint32_t* rot_list = nullptr;  // pcap: particles whose epilog rotation runs in k_epilog_rotation
  bool damp_stale = false;       // contact parameters changed since the list's per-pair damping was set
  // analysis (dem_set_analysis): per-interaction contact state, rcap entries
  bool analysis = false;
  dem::ContactStateArrays cs{};
  uint64_t cs_cap = 0;
  // multi-material contact parameters (dem_set_multimat); mm_pp == nullptr: singlemat
  int mm_ng = 0, mm_nd = 0;
  dem_contact_params* mm_pp = nullptr;  // device, mm_ng * mm_ng
  dem_contact_params* mm_pd = nullptr;  // device, mm_ng * mm_nd
  dem::ParamTable ptable() const {
    dem::ParamTable t;
    t.pp = mm_pp;
    t.pd = mm_pd;
    t.ng = mm_ng;
    t.nd = mm_nd;
    return t;
  }
  double* Dscr[7] = {};

  // scan scratch
  uint32_t* scan_blk = nullptr;
  uint64_t scan_cap = 0;

  // small device scalars: [0] displacement flag, [1] active contacts, [2] overflow
  unsigned long long* d_scalars = nullptr;
  unsigned long long* h_scalars = nullptr;  // pinned
  double* d_red = nullptr;                  // reduction scratch
  uint64_t red_cap = 0;

  uint64_t rebuilds = 0;
  uint64_t n_active = 0;

  // polyhedron mode (dem_set_shapes)
  bool poly = false;
  int nshapes = 0;
  int MV = 0;                         // max vertices of a shape (vertex stride)
  void* shapes_dev = nullptr;         // dem::ShapeDev[nshapes]
  double* vtx[3] = {};                // world vertices, n*MV each
  double* bvtx[3] = {};               // vertices at the last rebuild
  double* pobb = nullptr;             // world OBB per particle (15 doubles)
  float* vrf[3] = {};                 // FP32 vertices relative to the particle centre (rebuild time)
  float* vwf[3] = {};                 // FP32 roundings of the world vertices (every vertex computation)
  float* pfbox = nullptr;             // FP32 gate OBB + vertex slabs per particle (rebuild time)
  float4* pqb = nullptr;              // FP32 orientation backup (w, x, y, z) at the last rebuild
  uint32_t* vneed = nullptr;          // 1 for particles whose vertices the interaction list uses (n+1)
  uint32_t* vneed_off = nullptr;      // exclusive scan of vneed (n+1)
  uint32_t* vlist = nullptr;          // those particles, ascending
  uint64_t nvlist = 0;
  uint64_t vcap = 0;
  uint32_t* u_off = nullptr;          // n+1 unit offsets per owner
  uint32_t* urec = nullptr;           // 16 units per owner recorded by the unit count pass
  uint32_t* u_owner = nullptr;        // unit arrays (ucap each)
  uint32_t* u_partner = nullptr;
  uint64_t* u_pid = nullptr;
  uint32_t* u_kind = nullptr;
  uint8_t* u_pass = nullptr;
  uint16_t* u_slots = nullptr;        // features recorded by the count pass (FEAT_SLOTS per unit, or learned)
  uint64_t slot_cap = 0;              // entries of u_slots
  uint32_t* u_types = nullptr;        // exact VV, VE, VF, EE counts per unit (u8 x 4), count pass
  uint32_t* u_slotoff = nullptr;      // learned sizing: record offsets (ucap + 1)
  uint32_t* u_order = nullptr;        // learned sizing: count-pass order (warp bins)
  float* u_x = nullptr;               // MLP inputs per unit (16 floats)
  float* u_rates = nullptr;           // MLP rates per unit (4 floats)
  bool learned_slots = false;         // the current rebuild uses u_slotoff / u_order
  uint64_t learned_overflow = 0;      // units whose features overflowed the predicted record (last rebuild)
  uint64_t learned_units = 0;
  uint64_t nu_last = 0;               // units of the last polyhedron rebuild
  bool labels_valid = false;          // u_types holds the last rebuild's exact counts
  uint32_t* u_rec = nullptr;          // flattened enumeration: 16 words (masks, dR, S, R) per unit (ucap)
  uint32_t* t_cnt = nullptr;          // tests per (segment, unit), segment-major (6 ucap + 1); then kept tests
  uint32_t t_ntests = 0;              // tests of the last flattened count pass
  uint32_t* t_off = nullptr;          // their offsets (6 ucap + 1)
  uint32_t* t_keep = nullptr;         // kept bit per test (t_keepcap words)
  uint64_t t_keepcap = 0;
  bool t_flat = false;                // the last count pass was the flattened one
  uint32_t* f_cnt = nullptr;          // features per unit (ucap+1)
  uint32_t* f_off = nullptr;          // feature offsets (ucap+1)
  uint64_t ucap = 0;

  // inner bonds (k_bond.cu), double-buffered for the compaction at a rebuild
  uint64_t nb = 0, bcap = 0, nif = 0;
  dem::BondArrays B[2]{};
  void* bblock[2] = {nullptr, nullptr};
  int bcur = 0;
  uint32_t* b_scan = nullptr;        // bcap + 1: flags, then offsets
  uint32_t* b_iface = nullptr;       // bcap + 1: interface offsets
  uint64_t* bh_oid = nullptr;        // bcap: bonds broken since the last rebuild, as vertex-vertex history
  uint64_t* bh_pid = nullptr;
  uint32_t* bh_sub = nullptr;
  double* bh_ft[3] = {};
  uint64_t nbh = 0;
  uint32_t* b_own_first = nullptr;   // bpcap each: owned bonds of a slot
  uint32_t* b_own_cnt = nullptr;
  uint32_t* b_rev_off = nullptr;     // bpcap + 1: bonds where the slot is j
  uint32_t* b_rev_cur = nullptr;     // bpcap + 1
  uint32_t* b_rev_idx = nullptr;     // bcap
  uint32_t* b_inv = nullptr;         // bpcap: old slot -> new slot at a reorder
  uint64_t bpcap = 0;
  int ib_ng = -1;                    // -1: no inner bond parameters; 0: one set
  dem_inner_bond_params* ibp_dev = nullptr;
  std::vector<dem_inner_bond_params> ibp_host;
  std::vector<char> shapes_host;     // host copy of the dem::ShapeDev array (stick_polyhedra)

  // built-in profiler: launches always counted; CUDA-event times when enabled
  bool prof_on = false;
  uint64_t launches[K_NCLASS] = {};
  double prof_ms[K_NCLASS] = {};
  uint64_t prof_n[K_NCLASS] = {};
  struct PendingEv {
    int k;
    cudaEvent_t a, b;
  };
  std::vector<PendingEv> pending;
  std::vector<cudaEvent_t> ev_pool;
  cudaEvent_t get_event() {
    if (!ev_pool.empty()) {
      cudaEvent_t e = ev_pool.back();
      ev_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  void fold_events() {
    for (auto& p : pending) {
      float ms = 0.f;
      if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
        prof_ms[p.k] += ms;
        prof_n[p.k]++;
      }
      ev_pool.push_back(p.a);
      ev_pool.push_back(p.b);
    }
    pending.clear();
  }

  int fail(int code, const std::string& msg) {
    last_err = msg;
    return code;
  }
};

namespace dem {
// k_scan.cu
int scan_exclusive_u32(dem_ctx* c, const uint32_t* in, uint32_t* out, uint64_t n);
// k_grid.cu
int launch_bin_particles(dem_ctx* c);
int launch_reorder_particles(dem_ctx* c);
// k_neigh_sphere.cu
int launch_count_sphere(dem_ctx* c);
int refresh_pair_damp(dem_ctx* c);  // k_neigh_sphere.cu
int mark_records_live(dem_ctx* c);  // dem_api.cu
int ext_ensure_contact_state(dem_ctx* c);  // dem_api.cu: analysis arrays of the records' capacity
int launch_fill_sphere(dem_ctx* c, uint32_t* new_off, uint64_t total);
int launch_reverse_lists(dem_ctx* c);
// k_mesh.cu: bins of the mesh drivers for the current radius bound and skin
int ensure_mesh_bins(dem_ctx* c);
void free_meshes(dem_ctx* c);
int ext_add_driver(dem_ctx* c, const dem::DriverDev& d);  // dem_api.cu
// k_contact_sphere.cu
int launch_contact_sphere(dem_ctx* c);
int launch_gather_forces(dem_ctx* c);
// k_particles.cu
int launch_reset_force_moment(dem_ctx* c);
int launch_gravity(dem_ctx* c);
int launch_force_to_accel(dem_ctx* c);
int launch_prolog(dem_ctx* c);
int launch_epilog(dem_ctx* c);
int launch_displ_over(dem_ctx* c);
int launch_state(dem_ctx* c, dem_state* out);
int launch_profile(dem_ctx* c, int nslabs, double zlo, double zhi, double* out);
int launch_reciprocals(dem_ctx* c, uint64_t n);  // on P[0] after an upload
// k_poly.cu
int launch_poly_vertices(dem_ctx* c, int mode);  // 0 plain, 1 + displacement flag, 2 + backup & OBBs
int launch_poly_units(dem_ctx* c, uint64_t* nu_out, int (*grow_units)(dem_ctx*, uint64_t));
int launch_poly_feature_count(dem_ctx* c, uint64_t nu, uint32_t* total);
int launch_poly_feature_fill(dem_ctx* c, uint64_t nu);
int launch_contact_poly(dem_ctx* c);
int launch_state_systems(dem_ctx* c, dem_state* out);  // one state per system
void mlp_free(dem_ctx* c);
int mlp_rates(dem_ctx* c, const float* dev_x, uint64_t n, float* dev_rates);
int mlp_check(dem_ctx* c);
bool mlp_ready(const dem_ctx* c);
int launch_unit_features(dem_ctx* c, uint64_t nu);       // u_x of every unit
int launch_learned_sizing(dem_ctx* c, uint64_t nu);      // rates -> records, bins (host sync)
int launch_harvest(dem_ctx* c, float* x, uint8_t* y, uint64_t capacity, uint64_t* count, uint64_t* available);
int scan_reserve(dem_ctx* c, uint64_t n);
// graph step (dem_graph.cu) and the allocators it uses (dem_api.cu)
int step_graph(dem_ctx* c, int nsteps);
void free_graph(dem_ctx* c);
int ext_alloc_iarrays(dem_ctx* c, int b, uint64_t need);
int ext_alloc_records(dem_ctx* c, uint64_t need);
void ext_free_iarrays(IArrays& I);
int launch_poly_fused_prolog(dem_ctx* c);     // prolog + FP32-decided vertex_displ_over flag
int launch_vertex_list(dem_ctx* c);           // particles whose vertices the list uses (host sync)
int launch_poly_vertices_listed(dem_ctx* c);  // FP64 vertices of those particles
// k_bond.cu
int bonds_before_reorder(dem_ctx* c);  // rebuild: broken bonds -> history; interfaces
int bonds_after_reorder(dem_ctx* c);   // rebuild: new slots, per-slot bond lists
int launch_bond_criterion(dem_ctx* c); // ORs the rebuild flag when an interface breaks
int launch_bond_force(dem_ctx* c);     // bond pass + bond gather (after the contact gather)
int launch_bond_needs(dem_ctx* c, uint32_t* need);
void free_bonds(dem_ctx* c);
void clear_bonds(dem_ctx* c);
// k_step_fused.cu
int launch_fused_prolog(dem_ctx* c);
int launch_contact_compact(dem_ctx* c);
int launch_fused_epilog(dem_ctx* c);
}  // namespace dem

inline unsigned grid_for(uint64_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// RAII scope around the launches of one kernel class on the ctx stream.
struct ProfScope {
  dem_ctx* c;
  int k;
  cudaEvent_t a = nullptr;
  ProfScope(dem_ctx* ctx, int kclass, int nlaunch = 1) : c(ctx), k(kclass) {
    if (c->capturing) {  // counted per replay; no events inside a graph
      (c->capturing_body ? c->graph_launches_per_rebuild : c->graph_launches_per_step)[k] += (uint64_t)nlaunch;
      return;
    }
    c->launches[k] += (uint64_t)nlaunch;
    if (c->prof_on) {
      a = c->get_event();
      cudaEventRecord(a, c->stream);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEvent_t b = c->get_event();
      cudaEventRecord(b, c->stream);
      c->pending.push_back({k, a, b});
      if (c->pending.size() > 4096) c->fold_events();
    }
  }
};
