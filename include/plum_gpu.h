/* plum_gpu.h -- C ABI of the GB300 Monte Carlo energy engine.
 *
 * One context holds one system (or a batch of replicas) resident on one GPU:
 * bead positions, charges and types, the Ewald structure factor S(k), and the
 * running energy totals. Every entry point takes plain pointers and sizes;
 * host buffers are copied in and out by the call.
 *
 * The reference (nuwapi/Plum) has no FFI: its hot path sits behind C++ class
 * methods called by Simulation. Each entry point below replaces one of those
 * methods (file:line in the reference's src/ tree); the C++ host classes in
 * plum_gb300/csrc/host/ keep the reference's method names and call these.
 *
 * Error convention: every call returns PLUM_OK (0) or a PLUM_ERR_* code;
 * plum_last_error() returns a message for the calling thread. The reference
 * exits the process on bad input (e.g. simulation.cc:142-156, 594-597); this
 * library returns PLUM_ERR_INPUT instead. Energies keep the reference's 1e8
 * overlap sentinel (utilities/constants.h:15) and its "no Metropolis draw when
 * dE >= 1e8" rule (simulation.cc:327-332).
 *
 * Threading: a context binds one CUDA stream; calls on one context must not
 * overlap. Distinct contexts are independent.
 */
#ifndef PLUM_GPU_H_
#define PLUM_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLUM_OK 0
#define PLUM_ERR_INPUT 1     /* malformed or unsupported input */
#define PLUM_ERR_CUDA 2      /* a CUDA call failed */
#define PLUM_ERR_TIMEOUT 3   /* a device-side bounded wait gave up */
#define PLUM_ERR_NONFINITE 4 /* NaN/Inf energy detected on the device */
#define PLUM_ERR_STATE 5     /* call out of order (e.g. finalize without delta) */
#define PLUM_ERR_STREAM 6    /* recorded random stream exhausted */

/* Arithmetic of the pair and k-space sums. */
#define PLUM_FORM_FP64 0 /* plain form: FP64 everywhere (the drop-in) */
#define PLUM_FORM_FP32 1 /* precision form: FP32 pair/k arithmetic, FP64
                            S(k) and energy accumulators */

typedef struct plum_ctx plum_ctx;

typedef struct {
  int n_bead, n_mol, n_type, n_kvec; /* n_kvec: half-space k-vectors */
  int npbc, form;
  double box[3];      /* simulation box */
  double ewald_box[3]; /* Ewald box (z padded when the dipole correction is on) */
  double real_cutoff, kcut2, alpha, lB;
  int real_cell[3], k_cell[3];
} plum_info;

/* Run-control items of run.in (simulation.cc:30-50, force_field.cc:65-103). */
typedef struct {
  long steps, steps_eq, sample_freq, stat_out_freq, traj_out_freq;
  double beta, move_size, move_prob[5];
  int phantom, coion, grafted, grafted_counterion, calc_chem_pot;
  int use_pair, use_ewald, use_bond, use_bond_rigid, use_ext, use_gc, gc_freq;
  double rigid_bond, eq_bond;
  char run_name[256];
} plum_run_info;

/* Message for the last failing call on this thread ("" if none). */
const char* plum_last_error(void);

/* Creates a context from the reference's own inputs: `runin` (relative to
 * `dir`) in the positional grammar of simulation.cc:30-50 and
 * force_field.cc:64-195, plus the coordinate and topology files it names
 * (simulation.cc:582-646). Replaces Simulation::Simulation's reading and
 * ForceField::Initialize + InitializeEnergy (force_field.cc:46-405).
 * The total energy is computed on the device before returning. */
int plum_ctx_create(const char* dir, const char* runin, int form, int device,
                    plum_ctx** out);
/* Same, with the run.in content passed as text (the reference reads it from
 * stdin, simulation.cc:30-50); crd/top paths are relative to `dir`. */
int plum_ctx_create_text(const char* dir, const char* runin_text, int form, int device,
                         plum_ctx** out);
int plum_ctx_destroy(plum_ctx* ctx);
int plum_ctx_info(const plum_ctx* ctx, plum_info* out);
int plum_run_params(const plum_ctx* ctx, plum_run_info* out);
/* Molecule layout (n_mol+1 offsets), charges and type indices of the beads in
 * molecule order, as read from the coordinate file (simulation.cc:582-608);
 * any pointer may be NULL. */
int plum_get_topology(const plum_ctx* ctx, int* mol_start, double* q, int* type);
/* Bead symbol of a type index (first-appearance order in the crd file). */
int plum_type_name(const plum_ctx* ctx, int type, char* buf, int cap);

/* Recomputes every energy term of the current configuration from scratch on
 * the device in FP64 and resets the running totals and S(k) to it.
 * out[8] = {pair, ewald, bond, ext, ewald_real, ewald_recip, ewald_self,
 * ewald_dipole}. Replaces ForceField::InitializeEnergy
 * (force_field.cc:365-405) and the potentials' EnergyInitialization
 * (potential_pair.cc:55-100, potential_ewald.cc:176-231,
 * potential_bond.cc:16-27, potential_external.cc:48-61). */
int plum_total_energy(plum_ctx* ctx, double* out);

/* Running totals out[4] = {pair, ewald, bond, ext}. Replaces
 * ForceField::TotPairEnergy/TotEwaldEnergy/TotBondEnergy/TotExtEnergy
 * (force_field.cc:1201-1219). */
int plum_energies(const plum_ctx* ctx, double* out);

/* Energy difference of a trial configuration of molecule `mol`:
 * trial_xyz[size*3] and moved[size] (host buffers, the molecule's beads in
 * order). out[5] = {dE, dE_pair, dE_ewald, dE_bond, dE_ext}. The trial is
 * kept pending until plum_finalize. Replaces ForceField::EnergyDifference
 * (force_field.cc:407-434). */
int plum_delta_energy(plum_ctx* ctx, int mol, const double* trial_xyz,
                      const int* moved, double* out);

/* Accepts (commit trial, update S(k) and totals) or rejects the pending
 * trial. Replaces ForceField::FinalizeEnergies (force_field.cc:436-451) plus
 * the coordinate update of Simulation::TranslationalMove
 * (simulation.cc:336-351). */
int plum_finalize(plum_ctx* ctx, int accept);

/* Runs `n_moves` Monte Carlo steps entirely on the device: per step one draw
 * for the grand-canonical check (simulation.cc:221), molecule and move-type
 * choice, the trial move, dE and the Metropolis test, consuming the recorded
 * mt19937 output `stream[n_stream]` (host buffer) in the reference's draw
 * order. Replaces Simulation::Run's translational branch
 * (simulation.cc:216-355) with the Molecule moves (molecule.cc:103-312).
 * Optional per-step logs (host buffers of n_moves, may be NULL): move type
 * (0..4, -1 none), accept flag, total energy after the step.
 * *draws_used receives the number of stream words consumed. */
int plum_run_moves(plum_ctx* ctx, const uint32_t* stream, long n_stream,
                   int n_moves, int* move_type, int* accept, double* etot,
                   long* draws_used);
/* plum_run_moves with one more per-step log (host buffer of n_moves, may be
 * NULL): de[i] = the energy change ForceField::EnergyDifference
 * (force_field.cc:407-434) gives step i's proposal in the context's form (the
 * value the Metropolis test of simulation.cc:324-332 uses; >= 1e8 on
 * overlap), NaN for a step without a move. Two contexts of the same system in
 * the two forms fed the same stream propose the same moves until their first
 * differing decision, so their logs compare FP32 with FP64 energy changes
 * proposal by proposal on the chain's own moves. */
int plum_run_moves_de(plum_ctx* ctx, const uint32_t* stream, long n_stream,
                      int n_moves, int* move_type, int* accept, double* etot,
                      double* de, long* draws_used);

/* Same loop with the mt19937 stream generated on the device from `seed`
 * (std::mt19937 semantics) instead of a host buffer: the throughput path.
 * Continues the device generator across calls; plum_seed resets it. */
int plum_seed(plum_ctx* ctx, uint32_t seed);
int plum_run(plum_ctx* ctx, int n_moves, int* accepted_out);

/* Current coordinates, n_bead*3 doubles (host buffer), molecule order. */
int plum_get_positions(const plum_ctx* ctx, double* xyz);
/* Replaces the current coordinates (n_bead*3) and recomputes the energy. */
int plum_set_positions(plum_ctx* ctx, const double* xyz);

/* Snapshot of a context's step state for an exact restart (no reference
 * counterpart: the reference only writes its last coordinates): current
 * positions, running energies, S(k) with any pending update of the last
 * accepted move, per-molecule bond energies and the device counters.
 * plum_ctx_save copies it into a host buffer of plum_ctx_snapshot_size
 * bytes; plum_ctx_load restores it into a context created from the same
 * inputs and form (else PLUM_ERR_INPUT), after which the same draws
 * (plum_run_moves, or the host classes' generator) give bit-identical
 * steps. The device generator of plum_run is not part of it. No move may be
 * pending. */
long plum_ctx_snapshot_size(const plum_ctx* ctx);
int plum_ctx_save(const plum_ctx* ctx, void* buf, long size);
int plum_ctx_load(plum_ctx* ctx, const void* buf, long size);

/* The running Ewald structure factor S(k) = sum_i q_i e^{i k.r_i} over the
 * half-space k-set (plum_info.n_kvec vectors), with the change of the last
 * accepted move applied: sk_out[2 k + {0, 1}] = {Re, Im}, kn_out[3 k + a] =
 * the integer k components (k_a = 2 pi n_a / ewald_box[a]); either may be
 * NULL, nothing is written without Ewald. The reference keeps no S(k): its
 * reciprocal energy is a pairwise sum over the same k-set
 * (potential_ewald_coul.cc:198-225); plum_total_energy rebuilds S(k) from
 * scratch, so comparing the two checks the incremental updates. */
int plum_structure_factor(const plum_ctx* ctx, double* sk_out, int* kn_out);

/* out[5] = {Rg^2 averaged over chains, Rg_x^2, Rg_y^2, Rg_z^2, end-to-end^2}
 * of the current configuration. Replaces Simulation::RadiusOfGyration,
 * RadiusOfGyrationXYZ and EndToEndDistance (simulation.cc:406-500). */
int plum_observables(const plum_ctx* ctx, double* out);

/* The same per chain (molecules of more than one bead, in molecule order):
 * out[5 i + q] = {Rg^2, Rg_x^2, Rg_y^2, Rg_z^2, end-to-end^2} of chain i,
 * the terms plum_observables averages (simulation.cc:406-500). *n_chains
 * (may be NULL) receives the number of chains; at most cap chains are
 * written (cap = 0 only reports it). */
int plum_chain_observables(const plum_ctx* ctx, double* out, int cap, int* n_chains);

/* rho(z) of the current configuration, one sample of Simulation::CalcRhoZ
 * (simulation.cc:1029-1045): bins of 0.02 along z (z wrapped into [0, Lz)),
 * out[3*bin + id] with id 0 for chain beads, 1 for ions with q >= 0, 2 for
 * q < 0, each bead adding 1/(Lx Ly 0.02); molecules before `phantom` are
 * skipped. The reference accumulates samples into density_z_cumu; the
 * caller sums the returned samples. *n_bins (may be NULL) receives
 * ceil(Lz/0.02); at most cap values are written (cap = 0 only reports
 * n_bins). */
int plum_rhoz(const plum_ctx* ctx, double* out, int cap, int* n_bins);

/* The wall-force pressure sums of slit systems on the current configuration,
 * one evaluation of ForceField::CalcPressureForceLJELSlit (pressure.cc:404-488):
 * the z forces between the wall sites (the first `phantom` molecules' first
 * beads, half per wall) and the beads after them, LJ (PairForce) and Ewald
 * (PairForceZReal + PairForceZRepl), weighted -1/2, +1/2 and -1 as the
 * reference weights them, plus half of each system bead's external force
 * (BeadForceOnWall). out6 = the increments of p_tensor[6..11]: {LJ ions, LJ
 * polymers, LJ wall-wall, Ewald ions, Ewald polymers, Ewald wall-wall}. The
 * reference adds the wall-wall terms only on its first evaluation (the walls
 * do not move); the caller does the accumulating and averaging
 * (pressure.cc:471-487). The LJ force follows the reference's evident intent:
 * its PairForce reads an uninitialised local (potential_truncated_lj.cc:95-100).
 * PLUM_ERR_STATE while a trial move is pending. */
int plum_pressure_slit(plum_ctx* ctx, double* out6);

/* Configurational-bias trial-site energies of one growth step: for each of
 * n_trials trial positions b1[t] of the grand-canonical species' next bead
 * (and, for a charged species, its trial counterion b2[t]), the energy
 * ForceField::BeadsEnergy (cbmc.cc:5-151) returns: LJ and Ewald with the
 * system outside the molecules being deleted, with the chain_len beads grown
 * so far (chain, and their counterions chain_ci), with each other, self and
 * dipole terms and the walls; 1e8 on overlap. delete_mol is the molecule
 * being deleted (cbmc.cc:340-346; its counterions follow it), -1 when
 * inserting. Host buffers: b1, b2 [n_trials*3], chain, chain_ci
 * [chain_len*3], u_out [n_trials]. Used by CBMCFGenTrialBeads
 * (cbmc.cc:161-212), CBMCFChainInsertion and CBMCFChainDeletion
 * (cbmc.cc:214-442).
 *
 * The context's form picks the arithmetic: PLUM_FORM_FP64 in FP64 (three
 * launches); PLUM_FORM_FP32 in one launch with FP32 pair and k-space terms
 * on the fixed-point coordinates and FP64 sums across blocks (limits: the
 * trial sites and grown chain staged in at most 200 KiB of shared memory,
 * about 2,000 trials with a chain of 1,000; larger requests return
 * PLUM_ERR_INPUT). */
int plum_cbmc_trials(plum_ctx* ctx, int n_trials, const double* b1, const double* b2,
                     int chain_len, const double* chain, const double* chain_ci, int delete_mol,
                     double* u_out);

/* Device time of plum_cbmc_trials' kernels for these inputs: after three
 * untimed launches, `reps` launches between CUDA events on the context's
 * stream; ms_out = milliseconds per growth step, launches_out (may be NULL)
 * = kernel launches per growth step. No reference counterpart. */
int plum_cbmc_time(plum_ctx* ctx, int n_trials, const double* b1, const double* b2,
                   int chain_len, const double* chain, const double* chain_ci, int delete_mol,
                   int reps, double* ms_out, int* launches_out);

/* plum_cbmc_trials for callers that cannot allocate device memory: a host
 * application whose device memory is owned by its own allocator or budget,
 * or a grand-canonical driver that must not stall, since cudaMalloc and
 * cudaFree (which plum_cbmc_trials uses when a larger request grows its
 * buffers) synchronise the whole device. No counterpart in the reference.
 *
 * The energies are those of plum_cbmc_trials in the plain form: the FP64
 * kernels run whatever the context's form. They start from the context's
 * running S(k), which in a precision-form context carries the FP32 drift of
 * the moves since its last full recompute (none right after plum_ctx_create
 * or plum_total_energy). Every buffer is the caller's and is
 * in DEVICE memory: d_b1, d_b2 [n_trials*3], d_chain, d_chain_ci
 * [chain_len*3], d_u_out [n_trials]. The call allocates nothing (no
 * cudaMalloc/cudaFree, no host heap): its working memory is one fixed array
 * of 850 KiB inside the library, held on every GPU that loads the library
 * until the process exits. Limits: n_trials <= 256, chain_len <= 1024, at
 * most 32768 half-space k-vectors (the Ewald k-set of run.in); larger
 * requests return PLUM_ERR_INPUT. Nothing has to be zeroed first: each call
 * writes all the working memory it reads.
 *
 * The first call on each device does a one-time set-up (it looks up the
 * array's device address, with that device current): make that first call
 * on each device before any stream capture begins. All calls share the one
 * array, so calls that overlap on the GPU (from several threads or contexts
 * on the same device) race; serialise them. Every call ends by
 * synchronising the context's stream. Errors are returned as codes, with the message
 * written to err[err_cap] (may be NULL); plum_last_error is not updated. */
int plum_cbmc_trials_noalloc(plum_ctx* ctx, int n_trials, const double* d_b1,
                             const double* d_b2, int chain_len, const double* d_chain,
                             const double* d_chain_ci, int delete_mol, double* d_u_out,
                             char* err, int err_cap);

/* Grand-canonical parameters of run.in (force_field.cc:96-103): out9 =
 * {chem_pot, deBroglie prefactor, bead charge, chain length, CBMC trials,
 * GC frequency, spring constant, r0, type index of the species' beads}. */
int plum_gc_info(const plum_ctx* ctx, double* out9);
/* Appends n_mols molecules after the last one (as the reference's
 * mols.push_back on an accepted insertion, cbmc.cc:294-312): sizes[n_mols],
 * and for the sum of sizes beads xyz[3*n], q[n], type[n] (type indices of
 * plum_type_name). The running totals and S(k) are recomputed from scratch
 * (ForceField::EnergyInitForAddedMolecule, force_field.cc:1088-1105, updates
 * them incrementally; they agree to round-off). */
int plum_append_molecules(plum_ctx* ctx, int n_mols, const int* sizes, const double* xyz,
                          const double* q, const int* type);
/* Removes molecules [first, first + count) (simulation.cc:383-391 with the
 * potentials' AdjustEnergyUponMolDeletion); totals recomputed as above. */
int plum_erase_molecules(plum_ctx* ctx, int first, int count);

/* Full FP64 recompute cadence of plum_run, in moves (0 = never). The
 * precision form defaults to 10000: every 10^4 moves (at the next batch
 * boundary of 256) the totals, S(k) and the fixed-point mirror are rebuilt
 * from the FP64 positions, which resets FP32 drift. No reference counterpart
 * (the reference never recomputes, force_field.cc:1201-1219). */
int plum_set_recompute(plum_ctx* ctx, long every);
/* Drift found at the last recompute: out[5] = {pair, ewald, bond, ext}
 * running-minus-recomputed, and the largest |total drift| seen so far. */
int plum_drift(const plum_ctx* ctx, double* out);

/* Measured duration (ms) of the last plum_run/plum_run_moves call's device
 * work, and the number of kernels it launched. */
int plum_last_timing(const plum_ctx* ctx, double* ms, long* kernels);
/* n_moves more steps of plum_run as plain launches with CUDA events around
 * each kernel: out2 = mean milliseconds per launch of {energy change,
 * serial step}. For measurement; the steps count as ordinary steps. No
 * reference counterpart. */
int plum_time_kernels(plum_ctx* ctx, int n_moves, double* out2);

/* Measures the FP32 and FP64 FMA throughput of `device` (TFLOP/s, an FMA
 * counted as 2 FLOPs) with a short probe kernel: the roofline denominator of
 * the pair and k-space kernels, which run on the FP32/FP64 pipes rather than
 * the tensor cores. No reference counterpart. */
int plum_probe_peaks(int device, double* fp32_tflops, double* fp64_tflops);

/* ---------------------------------------------------------------- replicas
 * Many independent systems (replicas, of uneven size) advanced together on
 * one GPU in the precision form: per step every replica attempts one move;
 * one launch evaluates all replicas' energy differences from a shared item
 * list (pair and k-space work items of every replica's pending move), one
 * launch runs every replica's serial step (one block each). Replica r draws
 * from its own device mt19937 seeded seed + r. Batches of steps are replayed
 * as a CUDA graph. No reference counterpart: the reference runs one system
 * per process (simulation.cc:216-239). */
typedef struct plum_batch plum_batch;
int plum_batch_create(int n, const char* const* dirs, const char* const* runins, int form,
                      int device, plum_batch** out);
int plum_batch_destroy(plum_batch* batch);
int plum_batch_seed(plum_batch* batch, uint32_t seed);
/* Seeds replica r's generator with seeds[r]. */
int plum_batch_seed_each(plum_batch* batch, const uint32_t* seeds);
/* n_steps moves per replica; *accepted_out = accepted moves summed over
 * replicas. Includes the replicas' full FP64 recomputes that fall due
 * (plum_batch_set_recompute): their device time is part of
 * plum_batch_last_timing. */
int plum_batch_run(plum_batch* batch, int n_steps, long* accepted_out);
/* Full FP64 recompute cadence of the replicas, in moves per replica (0 =
 * never; default 10000, as plum_set_recompute for one system): after every
 * `every` of its moves (at the next boundary of the batch's 32-step graphs)
 * a replica's totals, S(k) and fixed-point mirror are rebuilt from its FP64
 * positions, which resets its FP32 drift. The replicas' cadences start at
 * staggered phases (replica r after r * every / R moves), so each batch of
 * steps recomputes its share of them. No reference counterpart (the
 * reference sums exact FP64 changes and never recomputes,
 * force_field.cc:436-451, 1201-1219). */
int plum_batch_set_recompute(plum_batch* batch, long every);
/* Drift found by the recomputes: out[6 * r + q] for replica r = {pair,
 * ewald, bond, ext running-minus-recomputed at its last recompute, the
 * largest |total drift| over its recomputes, the number of its recomputes}.
 * *count (may be NULL) = recomputes in the last plum_batch_run, *ms (may be
 * NULL) = their device time in milliseconds. */
int plum_batch_drift(plum_batch* batch, double* out, long* count, double* ms);
/* Running totals of every replica in one device gather and one copy:
 * out[4 * r + q] = {pair, ewald, bond, ext} of replica r (plum_energies of
 * each replica, ForceField::Tot*Energy, force_field.cc:1201-1219). */
int plum_batch_energies(plum_batch* batch, double* out);
int plum_batch_size(const plum_batch* batch);
/* The context of replica r (owned by the batch): energies, positions and
 * observables through the single-system calls above. */
int plum_batch_replica(plum_batch* batch, int r, plum_ctx** ctx);
int plum_batch_last_timing(const plum_batch* batch, double* ms, long* kernels);
/* n_steps more steps with plain launches and CUDA events around every
 * kernel: out4 = mean milliseconds per launch of {energy change (delta),
 * serial step, surrogate descriptor (with its smearing), surrogate
 * inference} (0 for kernels that did not run). For measurement; the steps
 * count as ordinary steps of the replicas. */
int plum_batch_time_kernels(plum_batch* batch, int n_steps, double* out4);
/* Work items of the batched energy change: (moved, other) pairs per pair
 * item (>= 1024, a multiple of 256; a pair item holds up to 32 moved beads
 * against item_pairs / 32 other beads, at least 256), k-vectors per k item
 * (64..256, or 512 / 1024: up to four per thread, the moved beads' phase
 * tables built once per item), the grid (0: 4 blocks per SM) and the register budget as
 * resident blocks per SM (2, 3 or 4). They change only the summation order
 * inside FP32 partials. */
int plum_batch_set_tune(plum_batch* batch, int item_pairs, int k_tile, int grid,
                        int min_blocks);
/* Times the energy-change kernel on these replicas (`steps` steps per
 * candidate, see plum_batch_time_kernels) for item sizes {4096, 8192, 16384,
 * 32768} x k tiles {128, 256, 512, 1024} x grids {2, 3, 4, 6, 8} blocks per
 * SM x register budgets {2, 3, 4} blocks per SM, keeps the fastest (then the
 * two pair loops of plum_batch_set_real_term at those sizes); out4 (may be
 * NULL) = the chosen {item_pairs,
 * k_tile, grid, min_blocks}. */
int plum_batch_autotune(plum_batch* batch, int steps, int* out4);
/* The pair loop of the batched energy change. table = 1 (the default where
 * it applies): for LJ + Ewald replicas whose real cut-off is at most half
 * the box, the table of h(u) = erfc(sqrt u)/sqrt u (cubic pieces, 32 per
 * octave of u, about 1e-7 relative below u = 4; erfc(sqrt(alpha) r)/r =
 * sqrt(alpha) h(alpha r^2)) staged in shared memory and the trial and current
 * evaluations of a pair done together, branch-free. table = 0: the loop of
 * one evaluation at a time, the term from the context's table in global
 * memory (or the FP32 erfc fit where a cut-off lies past the table).
 * PLUM_ERR_INPUT for table = 1 if a replica's alpha r_c^2 is past the table
 * (2^5). plum_batch_autotune keeps whichever is faster at the sizes it picks;
 * plum_batch_real_term reports the current choice. */
int plum_batch_set_real_term(plum_batch* batch, int table);
int plum_batch_real_term(const plum_batch* batch);
/* The h(u) table itself (host copy, built like the batch's): bins of 1/32
 * octave of the table variable u' = scale u from 2^-14 to 2^5, per bin a
 * cubic in w = f / 32 (f the bin-local fraction of u'), out[4 b + q] =
 * coefficient q of bin b, at most cap bins; returns the number of bins.
 * scale = 1, cut = 0: the universal table. A batch whose replicas share alpha
 * and r_c stages the cut table, scale = 16 / (alpha r_c^2) and cut = 16: h(u'
 * / scale) below u' = 16 and zero from there on, so the real-space cut-off is
 * the table's own. Returns -1 (last error set) for scale <= 0 or cut < 0. For checks of
 * its accuracy; no reference counterpart. */
int plum_h32_table(float* out, int cap, double scale, double cut);
/* The FP64 table every form's FP64 real-space term uses (erfc(sqrt(alpha)
 * r)/r = sqrt(alpha) h(alpha r^2), h(u) = erfc(sqrt u)/sqrt u): 32 bins per
 * octave of u from 2^-12 to 2^5, a degree-8 polynomial in the bin-local
 * y in [-1/2, 1/2) per bin, out[10 b + q] = coefficient q of bin b (q = 9
 * is 0), at most cap bins; returns the number of bins. About 2e-16
 * relative below u = 8. For checks of its accuracy; no reference
 * counterpart (the reference calls erfc, potential_ewald_coul.cc:134-164). */
int plum_h64_table(double* out, int cap);
/* The surrogate descriptor's cell lists (on by default for replicas of the
 * precision form periodic on every axis with at least 3 cells of 7.5 sigma
 * per axis). Off, every replica takes the all-pairs descriptor kernel; the
 * descriptors are the same integers either way. */
int plum_batch_set_cells(plum_batch* batch, int on);
/* Step chains per batch: 1 (default) or 2 -- the replicas split in halves
 * whose chains run as two branches of the batch's graph on two streams, so
 * one half's latency-bound kernels overlap the other half's energy change.
 * Results are the same either way (each replica's arithmetic is unchanged). */
int plum_batch_set_groups(plum_batch* batch, int groups);
/* Capacity of the descriptor cell lists' list of beads that changed cell
 * since the last rebuild (reallocates the lists). When it overflows, that
 * replica takes the all-pairs descriptor kernel until the next batch of
 * steps, and the capacity doubles. */
int plum_batch_set_cell_cap(plum_batch* batch, int cap);
/* out4 = {replicas with a descriptor cell list, of which valid (no overflow
 * since the last rebuild), most beads in one replica's list of beads that
 * changed cell, its capacity}. For diagnostics. */
int plum_batch_cell_stats(plum_batch* batch, int* out4);
/* The descriptors of the replicas' last surrogate moves, out[R * 96] (the
 * rows stay as they were for replicas whose last move was not one). */
int plum_batch_descriptors(plum_batch* batch, float* out);

/* ---------------------------------------------------------------------
 * Learned surrogate and delayed acceptance. No counterpart in the
 * reference: an addition that keeps the stationary distribution of its
 * Metropolis step (simulation.cc:324-332).
 *
 * Descriptor of a move of beads [b_lo, b_hi) (96 values): 4 channels x 24
 * Gaussian-smeared radial bins (width 0.25 sigma, centres 0.125..5.875
 * sigma; pairs up to 7.5 sigma) of the pairs (moved bead, other bead; moved
 * pairs once): channel 0 neighbours of the moved bead's type before the
 * move, 1 other types before, 2 and 3 the same after the move. Values are
 * sums in units of 2^-12.
 *
 * Network: 96 -> 128 -> 128 -> 1, SiLU, BF16 weights, FP32 accumulation,
 * input standardised by (x - mu) * isd. Its surrogate energy change is
 * s = y_scale (f(x) - f(swap x)), swap exchanging channels (0,1) with (2,3),
 * so s of the reverse move is exactly -s. Parameters (fp32, in this order):
 * W1 [128][96], b1 [128], W2 [128][128], b2 [128], w3 [128], b3. */
typedef struct plum_surrogate plum_surrogate;
int plum_surrogate_nparams(void);
/* Glorot-uniform weights from seed, zero biases, mu = 0, isd = 1. */
int plum_surrogate_create(int device, unsigned long long seed, plum_surrogate** out);
int plum_surrogate_destroy(plum_surrogate* sg);
int plum_surrogate_set_params(plum_surrogate* sg, const float* params);
int plum_surrogate_get_params(const plum_surrogate* sg, float* params);
int plum_surrogate_set_norm(plum_surrogate* sg, const float* mu, const float* isd,
                            float y_scale);
/* Delayed acceptance uses s' = sign(s) max(|s| - margin, 0) (default 0):
 * still antisymmetric, so still exact; stage one then only rejects moves
 * predicted to cost more than `margin` k_BT. */
int plum_surrogate_set_margin(plum_surrogate* sg, float margin);
/* s for n descriptors x [n][96] (host buffers; _device: device buffers). */
int plum_surrogate_predict(plum_surrogate* sg, const float* x, long n, float* s_out);
int plum_surrogate_predict_device(plum_surrogate* sg, const float* d_x, long n, float* d_s);
/* Gradient of mean_n (s - t)^2 over every parameter, then the loss:
 * grad_out [nparams + 1] (host buffers). */
int plum_surrogate_grad(plum_surrogate* sg, const float* x, const float* t, long n,
                        float* grad_out);
/* Adam (beta 0.9, 0.999, eps 1e-8) with the given gradient [nparams]. */
int plum_surrogate_adam_step(plum_surrogate* sg, const float* grad, float lr);
/* Adam training on DEVICE data d_x [n][96], d_t [n]: `epochs` shuffled
 * passes (seeded) of n / batch steps; loss_out[epochs] (may be NULL) gets
 * each pass's mean loss. */
int plum_surrogate_train(plum_surrogate* sg, const float* d_x, const float* d_t, long n,
                         int batch, int epochs, float lr, unsigned long long seed,
                         double* loss_out);
/* Descriptor [96] of the pending trial move of plum_delta_energy (before
 * plum_finalize), in the units above. */
int plum_move_descriptor(plum_ctx* ctx, double* out);
/* Training data from the plain step loop (plum_run semantics, n_moves
 * steps): for each pivot, crankshaft or reptation move, its descriptor and
 * its exact energy change (1e8 on overlap) into DEVICE buffers d_desc
 * [cap][96] and d_de [cap]; *n_logged = rows written (at most cap). */
int plum_collect_surrogate_data(plum_ctx* ctx, int n_moves, long cap, float* d_desc,
                                double* d_de, long* n_logged);
/* Delayed acceptance in the replica batch (sg NULL turns it off; sg must
 * outlive its use). A chain move draws u1 after its own draws and is
 * rejected at stage one unless u1 < exp(-beta s); a move that passes draws
 * u2 and is accepted if u2 < exp(-beta (dE - s)) (no draw when dE >= 1e8).
 * Moves rejected at stage one skip the exact energy change. */
int plum_batch_set_surrogate(plum_batch* batch, const plum_surrogate* sg);
/* Totals since plum_batch_set_surrogate: out3 = {surrogate moves, stage-one
 * passes, accepted}. */
int plum_batch_da_stats(plum_batch* batch, long* out3);

#ifdef __cplusplus
}
#endif
#endif
