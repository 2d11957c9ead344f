// Device-side layout of one Monte Carlo system and the kernel entry points.
//
// HBM layout (one system, FP64 form):
//   pos    double4_32a[n_bead]  current (x, y, z, q), unwrapped coordinates
//   trial  double4_32a[n_bead]  trial   (x, y, z, q); equals pos outside the
//                           moved bead range of the pending move
//   type   int[n_bead]      bead type (index into the per-type tables)
//   mol_start int[n_mol+1]  beads of molecule m are [mol_start[m], mol_start[m+1])
//   kn     short4[n_k]      integer k = (nx, ny, nz) of each half-space vector
//   kw     double[n_k]      e^{-k^2/4a}/k^2 on the reference's k-set
//   sk     double2[n_k]     running structure factor S(k) = sum q e^{i k.r}
//   dsk    double2[2*n_k]   S(k) change of the pending move (double-buffered:
//                           an accepted change is added to sk by the next
//                           delta kernel)
//   partial double[grid*4]  per-block partial sums of the pending move
//   dsk_part double2[groups*n_k], kpartial double[k tiles]: k-space parts
//   state  DevState         running energies, the pending move, stream cursor
// Everything here is a few MB even at 20,000 beads and 15,624 k-vectors, so
// it stays L2-resident across moves; the pair sweeps are FP64/FP32-pipe
// bound, not HBM bound.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace plum {

constexpr int kMaxTypes = 8;
constexpr int kMaxT2 = kMaxTypes * kMaxTypes;
constexpr double kVeryLarge = 1e8;   // utilities/constants.h:15
constexpr double kRhoZRes = 0.02;    // density_z_res (simulation.cc:113)
constexpr double kPiRef = 3.14159265359;  // utilities/constants.h:20
constexpr double kMtMax = 4294967295.0;   // std::mt19937::max()

// Threads per block of the pair sweep.
constexpr int kPairThreads = 256;
constexpr int kMaxKmax = 1024;       // |n| per axis supported by the k tables
constexpr int kKTableBytes = 96 * 1024;  // shared memory budget for phase tables
constexpr int kSerialThreads = 256;
constexpr int kDrawWindow = 1024;    // stream words staged per serial launch

// Device-side error codes (same values as PLUM_ERR_* in include/plum_gpu.h).
constexpr int PLUM_ERR_TIMEOUT_DEV = 3;
constexpr int PLUM_ERR_NONFINITE_DEV = 4;
constexpr int PLUM_ERR_STREAM_DEV = 6;

struct DevParams {
  int n_bead, n_mol, n_type, npbc;
  int phantom, grafted, n_chain_total, n_ion_total;  // chain/ion pick lists
  double box[3], inv_box[3];
  double ebox[3], inv_ebox[3];
  int use_pair, use_ewald, use_bond, use_rigid, use_ext, dipole;
  double beta, move_size, move_prob[5];
  double bond_len;   // r0 (bond potential) or the rigid length
  int vary_bond;     // bond potential on: +-10% bond length draws
  // LJ per ordered type pair k = ti*n_type+tj (potential_truncated_lj.cc:49-85)
  double lj_sig2[kMaxT2], lj_eps4[kMaxT2], lj_rc2[kMaxT2], lj_eref[kMaxT2];
  // Ewald (potential_ewald_coul.cc:29-115)
  double lB, sqrt_alpha, real_cut;
  int real_cell[3];
  int single_image;  // real_cut <= half of every Ewald box length
  int n_k, kmax[3];
  int koff[3], kper;  // per-bead table: axis a at koff[a], n = 0..kmax[a]; kper entries
  int kchunk_delta, kchunk_sk;  // beads per table chunk (fits kKTableBytes)
  double kunit[3];   // 2 kPi / ebox[a]
  double kpref;      // lB/(kPi V) * 4 kPi^2
  double self_coef;  // -lB sqrt(alpha/kPi)
  double dip_coef;   // lB * 2 kPi / V
  // pair_kind 1: hard spheres (potential_hard_sphere.cc:38-49): overlap when
  // r <= hs_sum[k] (radius sum of the type pair); bonded neighbours of a
  // chain are skipped (potential_pair.cc:64-67, 163-167). The LJ tables then
  // hold lj_rc2 = a bound just above hs_sum^2 for the pre-tests.
  int pair_kind;
  double hs_sum[kMaxT2];
  float f_hs_sum[kMaxT2];
  // ext_kind 1: hard wall, 2: square-well wall (potential_hard_wall.cc:36-47,
  // potential_well_wall.cc:41-55), radius per type
  int ext_kind;
  double wall_rad[kMaxTypes], well_width, well_depth;
  // bonds (potential_spring.cc:22-48)
  double k_bond, r0;
  // walls (potential_truncated_lj_wall.cc:46-134)
  double wall_cut, wall_sig[kMaxTypes], wall_eps[kMaxTypes];
  int graft[kMaxTypes];
  // precision form (FP32 pair and k-space arithmetic)
  int form;              // 0 FP64, 1 FP32
  float f_scale[3];      // Ewald box length / 2^32: fixed-point unit per axis
  float f_box[3];        // Ewald box lengths
  float f_lj_sig2[kMaxT2], f_lj_eps4[kMaxT2], f_lj_rc2[kMaxT2], f_lj_eref[kMaxT2];
  float f_real_cut, f_sqrt_alpha, f_lB;
  double inv_fix[3];     // 2^32 / Ewald box length (FP64 -> fixed point)
  // cell list of the surrogate descriptor (replica batches, precision form,
  // periodic on every axis): cell_nc cells per axis, each at least the
  // descriptor's cut wide; cell_cap entries in the list of beads that left
  // their cell since the last rebuild (0: no cell list)
  int cell_nc[3], cell_cap;
  // FP32 h(u) table of the real-space term (kH32Bins entries, device memory;
  // null when alpha r_c^2 lies past it: the FP32 erfc fit is used then)
  const float4* htab;
  // FP64 h(u) table (kH64Bins x kH64Stride doubles; null: erfc / r), alpha
  // itself, and whether the pair box and the Ewald box wrap every periodic
  // axis alike (then one minimum-image vector serves LJ and Ewald)
  const double* htab64;
  double alpha;
  int same_wrap;
  double lj_max2;  // largest lj_rc2 over the type pairs in use
};

// The pending move: beads [b_lo, b_hi) of molecule `mol` hold trial
// positions in `trial`.
struct DevState {
  double e_pair, e_ewald, e_bond, e_ext;
  double mz;         // sum q z over the current configuration
  double dipl_cur;   // dipole energy as last committed (reference semantics)
  // pending move
  int pending, mol, b_lo, b_hi, move_type, step, step_open;
  // results of the last energy difference
  double de, de_pair, de_ewald, de_bond, de_ext, bond_trial, dipl_trial, dmz;
  int last_accept;
  // stream cursor
  long long stream_pos, stream_len;
  int error;         // PLUM_ERR_* raised on the device
  int moves_left;
  int n_accept;
  int n_nonfinite;   // steps whose dE was NaN/Inf (rejected, as in the reference)
  // pending move's sums, reduced by the last block of the delta kernel
  double red_lj, red_re, red_k;
  // S(k) commit of an accepted move is applied by the next delta kernel's
  // k tiles: dsk[sk_buf] is pending while sk_pending; the delta kernel writes
  // the new dS(k) into dsk[cur_buf]
  int sk_pending, sk_buf, cur_buf;
  // delayed acceptance (surrogate stage one before the exact energy change):
  // da_on enables it for chain moves; da_active marks the pending move as a
  // surrogate move, da_u1 is its stage-one draw, da_s the surrogate energy
  // change, da_skip the stage-one rejection (the exact change is not
  // computed). Counters: surrogate moves, stage-one passes, accepts.
  int da_on, da_active, da_skip, da_n_moves, da_n_pass, da_n_accept;
  double da_u1, da_s;
  // the descriptor's cell list holds every bead (cleared when a cell
  // overflowed: the all-pairs descriptor kernel then takes the replica
  // until the next rebuild)
  int cell_ok;
  // training log of (descriptor, exact dE) for surrogate moves (log_desc set)
  int log_n, log_cap;
};

// The fixed-point pair form of the FP64 kernels (k_delta64, k_total64):
// LJ + Ewald in a cubic box periodic on every axis, one image (r_c <= L/2),
// one box for both terms, the FP64 h(u) table.
__host__ __device__ inline bool fix_pairs(const DevParams& P) {
  return P.use_ewald && P.htab64 && P.same_wrap && P.npbc == 3 && P.single_image &&
         P.pair_kind == 0 && P.ebox[0] == P.ebox[1] && P.ebox[1] == P.ebox[2];
}

struct DevBuffers {  // all pointers: copied word-wise into shared memory by the batch kernels
  double4_32a* pos;
  double4_32a* trial;
  int* type;
  int* mol_start;
  int* chain_ids;
  int* ion_ids;
  short4* kn;
  double* kw;
  double2* sk;
  double2* dsk;      // [2][n_k] double-buffered dS(k)
  double* partial;   // [grid][4]
  // plain form mirror (fix_pairs systems; null otherwise): 64-bit
  // fixed-point fractions of the box (X, Y, Z) and the charge's bits
  ulonglong4_32a* fpos64;  // [n_bead] current positions
  // precision form mirrors: 32-bit fixed-point fractions of the Ewald box
  int4* fpos;        // [n_bead] current (X, Y, Z, type)
  float* fq;         // [n_bead] charges
  int4* ftrial;      // [max molecule length] trial of the pending move's beads
  float2* dsk_part32;  // [groups][n_k]
  double2* dsk_part; // [groups][n_k] dS(k) parts of the pending move
  int* ktile_count;  // [k tiles] arrival tickets (reset by the last arrival)
  int* done_count;   // [1] block arrival ticket of the delta kernel
  double* kpartial;  // [k tiles] energy change per k tile
  double* bond_mol;  // [n_mol]
  DevState* state;
  const uint32_t* stream;
  // per-step logs (may be null)
  int* log_type;
  int* log_accept;
  double* log_etot;
  double* log_step_de;  // energy change of each step's proposal (NaN: none)
  // surrogate: descriptor of the pending move [96] (integer units of
  // 2^-12), its fine distance histogram, and the optional training log
  unsigned* desc_acc;
  unsigned* desc_fine;  // [4][241] pair counts per 1/32-sigma distance bin
  float* log_desc;   // [log_cap][96]
  double* log_de;    // [log_cap]
  // descriptor cell list (null when the replica has none), rebuilt by a
  // counting sort: cell_ent [n_bead] holds (X, Y, Z, bead << 3 | type) sorted
  // by cell, cell c's entries at [cell_start[c], cell_start[c + 1]). An
  // accepted bead rewrites its entry in place while it stays in its cell;
  // when it leaves, the entry goes dead (w = -1) and the bead moves to
  // cell_extra [cell_cap] (cell-less, counted in cell_n[cells]), where it
  // stays until the next rebuild. cell_key: the bead's entry, k >= 0 in
  // cell_ent or -2 - e in cell_extra.
  int* cell_key;     // [n_bead]
  int* cell_n;       // [cells + 1] counts / cursors of the sort; [cells]: extra used
  int* cell_start;   // [cells + 1]
  int4* cell_ent;    // [n_bead]
  int4* cell_extra;  // [cell_cap]
};

// Wall-force pressure of slit systems (kern_pressure.cu, slit_pressure.h):
// partial-sum block counts for n_items pair + wall items and n_k k vectors
// (returns the scratch doubles needed), and the three launches; the six sums
// land at scratch[6 n1 + 3 n2 ..].
struct SlitPressParams;
int slit_partials_count(long long n_items, int n_k, int* n1, int* n2);
void launch_slit_pressure(const SlitPressParams& S, const DevBuffers& B, long long n_pair,
                          long long n_wall, int wall_b0, int n_k, const double* kunit,
                          double* scratch, int n1, int n2, cudaStream_t s);

// Launch helpers (kern_energy.cu / kern_moves.cu). All enqueue on `s`.
int pair_grid();
int ktile_count(const DevParams& P);
void launch_delta_pairs64(const DevParams& P, const DevBuffers& B, cudaStream_t s);
void launch_total64(const DevParams& P, const DevBuffers& B, double* out_partials,
                    int n_part, cudaStream_t s);
int total_partials_count(const DevParams& P);
// S(k) from scratch; part: sk_full_groups() * n_k double2 of scratch owned by
// the caller (one per context, so contexts on different streams never share it)
int sk_full_groups(const DevParams& P);
void launch_sk_full64(const DevParams& P, const DevBuffers& B, double2* part, cudaStream_t s);
void launch_misc_total64(const DevParams& P, const DevBuffers& B, double* out6,
                         cudaStream_t s);

// Serial step: mode bits
constexpr int kModeFinish = 1;   // reduce partials, compose dE
constexpr int kModeDecide = 2;   // Metropolis draw from the stream + commit
constexpr int kModeGen = 4;      // generate the next move from the stream
constexpr int kModeCommit = 8;   // commit/reject by state->last_accept (host decided)
void launch_serial64(const DevParams& P, const DevBuffers& B, int mode, cudaStream_t s);
void launch_set_move(const DevBuffers& B, int mol, int b_lo, int b_hi, cudaStream_t s);
void launch_observables64(const DevParams& P, const DevBuffers& B, double* per_mol,
                          double* out5, cudaStream_t s);
void launch_rhoz(const DevParams& P, const DevBuffers& B, double res, int n_bins, unsigned* cnt,
                 cudaStream_t s);
// precision form (kern_fp32.cu)
int pair_grid32();
void launch_delta_pairs32(const DevParams& P, const DevBuffers& B, cudaStream_t s);
// the plain form's 64-bit position mirror (B.fpos64), where it has one
void launch_fix64_all(const DevParams& P, const DevBuffers& B, cudaStream_t s);
void launch_fix_all(const DevParams& P, const DevBuffers& B, cudaStream_t s);
void launch_fix_trial(const DevParams& P, const DevBuffers& B, cudaStream_t s);

// configurational-bias trial sites (kern_cbmc.cu)
struct CbmcJob {
  int n_trials, charged, cl, type;  // trials, counterion present, grown beads, species type
  int ex_lo, ex_hi;                 // system beads of the molecules being deleted
  const double4_32a* b1;            // [n_trials] trial beads (x, y, z, q)
  const double4_32a* b2;            // [n_trials] trial counterions
  const double4_32a* chain;         // [cl] grown beads
  const double4_32a* chain_ci;      // [cl] their counterions
  double2* s_o;                     // [n_k] scratch: S(k) of the other charges
  double* part;                     // [n_trials][groups][2] scratch
  double* u;                        // [n_trials] result
};
int cbmc_groups(const DevParams& P);
void launch_cbmc(const DevParams& P, const DevBuffers& B, const CbmcJob& J, cudaStream_t s);
// The precision form's one-launch trial kernel (kern_cbmc32.cu): J.part holds
// `slots` doubles laid out by cbmc32_layout; J.s_o is unused. ticket is one
// int, zero before the first launch (each launch leaves it zero).
struct Cbmc32Layout {
  int n_grp, n_chunk, chunk, n_pair, n_kt, grid;
  long long chain_off, k_off, slots;
  size_t smem;
};
Cbmc32Layout cbmc32_layout(const DevParams& P, int n_trials, int chain_len);
size_t cbmc32_max_smem();
int launch_cbmc32(const DevParams& P, const DevBuffers& B, const CbmcJob& J,
                  const Cbmc32Layout& G, int* ticket, cudaStream_t s);
// The same on a fixed scratch array (no allocation); returns 0, 1 (sizes) or 2
// (CUDA), with a message in err.
int cbmc_trials_noalloc(const DevParams& P, const DevBuffers& B, cudaStream_t s, int device,
                        int n_trials, const double* d_b1, const double* d_b2, int chain_len,
                        const double* d_chain, const double* d_chain_ci, int type, int charged,
                        double q1, double q2, int ex_lo, int ex_hi, double* d_u, char* err,
                        int err_cap);

// batched replicas (kern_fp32.cu / kern_moves.cu)
constexpr int kMaxReplicas = 2048;
// Work-item sizes of the batched energy change (k_tile <= kPairThreads).
struct BatchTune {
  int item_pairs;  // (moved, other) pairs per pair item
  int k_tile;      // k-vectors per k item
  int grid;        // blocks (0: 4 per SM)
  int min_blocks;  // register budget: 2 or 3 resident blocks per SM
  int htab;        // real-space term from the h(u) table (1) or the erfc fit (0)
};
// FP32 table of h(u) = erfc(sqrt u) / sqrt u, the real-space Ewald term
// erfc(sqrt(alpha) r) / r = sqrt(alpha) h(alpha r^2) as a function of the
// dimensionless u = alpha r^2 alone, so one table serves every system. Bins:
// kH32Per per octave of u for octaves 2^kH32ELo .. 2^(kH32EHi - 1); bin b
// holds a cubic in w = f / 32, f in [0, 1) the bin-local fraction of u
// (its float mantissa bits below the top five).
// Built on the host by
// Chebyshev interpolation of std::erfc in double precision (build_h32_table).
// A cut table (scale s, cut c) tabulates h(u' / s) in the variable u' = s u
// and is zero on every bin at or above u' = c, a power of two and so a bin
// edge: with s = c / (alpha r_c^2) the cut-off of the real-space term is the
// table's own (the batched pair sweep of replicas sharing alpha and r_c).
constexpr int kH32ELo = -14, kH32EHi = 5, kH32Per = 32;
constexpr int kH32Bins = (kH32EHi - kH32ELo) * kH32Per;
constexpr double kH32Cut = 16.0;
void build_h32_table(float4* out, double scale = 1.0, double cut = 0.0);  // kH32Bins entries
// The FP64 table of h(u): kH64Per bins per octave of u for octaves
// 2^kH64ELo .. 2^(kH64EHi - 1), a degree-8 polynomial in y = f - 1/2 per bin
// (kH64Stride doubles per bin, the last zero, for 16-byte loads): Chebyshev
// interpolation of erfcl at 9 nodes in long double, converted to powers of y.
// About 2e-16 relative below u = 8; above it h < 3e-5 and the absolute error
// stays below 1e-17. u below the table takes erfc / r directly.
constexpr int kH64ELo = -12, kH64EHi = 5, kH64Per = 32, kH64Stride = 10;
constexpr int kH64Bins = (kH64EHi - kH64ELo) * kH64Per;
void build_h64_table(double* out);  // kH64Bins * kH64Stride entries
constexpr int kMinItemPairs = 1024;  // smallest item the slot buffers are sized for
constexpr int kMinKTile = 64;
// Pair items of the batched energy change: up to kPairGroup moved beads
// (staged in shared memory) x a chunk of other beads (one per thread, a
// multiple of the block size); one more item per move takes the pairs among
// the moved beads.
constexpr int kPairGroup = 32;
// Other beads per pair item: item_pairs over the staged group, the group
// counted as the table loop stages it (padded to a multiple of 4), so that an
// item of a one-bead move is no longer than a chain move's.
__host__ __device__ inline int pair_chunk(int m, int item_pairs) {
  const int g = m < kPairGroup ? ((m > 0 ? m : 1) + 3) & ~3 : kPairGroup;
  const int c = (item_pairs / g + kPairThreads - 1) / kPairThreads * kPairThreads;
  return c > kPairThreads ? c : kPairThreads;
}
__host__ __device__ inline int pair_item_count(int m, int n_bead, int item_pairs) {
  if (m <= 0) return 0;
  const int c = pair_chunk(m, item_pairs);
  return ((m + kPairGroup - 1) / kPairGroup) * ((n_bead + c - 1) / c) + (m > 1 ? 1 : 0);
}
// queue: two ints, zero before the first launch (each launch leaves them zero)
// htab: the universal table (cut_scale 0) or the batch's cut table (scale
// cut_scale = kH32Cut / (alpha r_c^2), every replica with the same alpha and r_c)
void launch_batch_delta32(const DevParams* rp, const DevBuffers* rb, int n_rep, int* item_off,
                          double* slots, size_t smem, BatchTune tune, int* queue,
                          const float4* htab, float cut_scale, cudaStream_t s);
void launch_batch_serial(const DevParams* rp, const DevBuffers* rb, const int* item_off,
                         const double* slots, int n_rep, int mode, cudaStream_t s);
// per replica r: if need[r], shift the unread words [pos[r], len[r]) of out[r]
// to the front and fill the rest up to cap[r] from state[r] (625 words)
void launch_mt_fill_batch(uint32_t* const* states, uint32_t* const* outs, const long long* pos,
                          const long long* len, const long long* cap, const int* need,
                          DevState* const* sts, int n_rep, cudaStream_t s);
void launch_gather_states(DevState* const* sts, int n_rep, long long* out, cudaStream_t s);
void launch_gather_energies(DevState* const* sts, int n_rep, double* out, cudaStream_t s);

// mt19937 on the device: state[625] (624 words + index), fills out[n].
void launch_mt_fill(uint32_t* state, uint32_t* out, long long n, cudaStream_t s);

}  // namespace plum

static_assert(sizeof(plum::DevParams) % sizeof(int) == 0, "DevParams is copied as ints");
static_assert(sizeof(plum::DevBuffers) % sizeof(long long) == 0, "DevBuffers is copied as 8-byte words");
static_assert(sizeof(plum::DevState) % sizeof(int) == 0, "DevState is copied as ints");
