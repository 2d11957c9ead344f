/* FP64 CPU restatement of the reference's Monte Carlo energy path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle: tests/, the smoke check and
 * bench.py's CPU-baseline leg load it as a checker. The product (plum_gb300)
 * never links, loads or calls it.
 *
 * It restates, in plain C and in the reference's FP64 arithmetic:
 *   - input readers     simulation.cc:23-50, 582-646; force_field.cc:64-195;
 *                       potential_truncated_lj.cc:20-47; potential_ewald_coul.cc:29-37;
 *                       potential_spring.cc:11-20; potential_truncated_lj_wall.cc:13-44
 *   - Ewald set-up      potential_ewald_coul.cc:38-115 (cutoffs, cells, k-set)
 *   - pair LJ           potential_truncated_lj.cc:49-85 with bead.cc:162-176
 *   - Ewald real        potential_ewald_coul.cc:134-164 with misc.cc:43-56
 *   - Ewald reciprocal  potential_ewald_coul.cc:198-225 rewritten as the
 *                       structure factor S(k) over the same k-set (half space)
 *   - self / dipole     potential_ewald_coul.cc:253-257, 415-428
 *   - bonds             potential_spring.cc:22-48, 63-80
 *   - walls             potential_truncated_lj_wall.cc:46-134; potential_external.cc:100-117
 *   - ForceField::EnergyDifference / FinalizeEnergies  force_field.cc:407-451
 *   - moves             molecule.cc:103-312; misc.cc:95-134
 *   - step loop         simulation.cc:216-355
 *   - observables       simulation.cc:406-500, 1029-1045
 */
#ifndef PLUM_ORACLE_H_
#define PLUM_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct po_ctx po_ctx;

/* Reads dir/runin plus the crd/top files it names (paths relative to dir).
 * Returns NULL and writes a message into err (cap bytes) on bad input. */
po_ctx* po_create(const char* dir, const char* runin, uint32_t seed, char* err,
                  int cap);
void po_destroy(po_ctx* c);
/* When on, po_create skips the O(N^2) pair and real-space totals (their
 * running values start at 0); S(k), bonds, walls and self terms are still
 * built. For timing moves on systems too large for an all-pairs sum. */
void po_set_fast_init(int on);

int po_n_bead(const po_ctx* c);
int po_n_mol(const po_ctx* c);
int po_n_kvec(const po_ctx* c);
/* out = {real_cutoff, kc2, real_cell[3], k_cell[3], ebox[3], alpha, lB, evol,
 *        dipole} (same layout as the reference harness' pr_ewald_info). */
void po_ewald_info(const po_ctx* c, double* out);

/* Energies of the current configuration recomputed from scratch:
 * out = {pair, ewald, bond, ext, ewald_real, ewald_recip, ewald_self,
 *        ewald_dipole}. Also resets the running totals and S(k). */
void po_total_energy(po_ctx* c, double* out);
/* Running totals {pair, ewald, bond, ext}. */
void po_energies(const po_ctx* c, double* out);

/* Delta energy of a trial configuration of molecule `mol` (trial: size x 3,
 * moved: size flags) as ForceField::EnergyDifference computes it, without
 * committing. out = {dE, dE_pair, dE_ewald, dE_bond, dE_ext}. */
void po_delta_energy(po_ctx* c, int mol, const double* trial, const int* moved,
                     double* out);

/* n reference steps (simulation.cc:220-229). Per step: move type (0..4, -1 if
 * nothing attempted), accept flag, draws consumed, running total energy. */
int po_run(po_ctx* c, int n, int* move_type, int* accept, int* draws,
           double* etot);
/* Same loop driven by an external recorded stream of mt19937 outputs instead
 * of the internal generator; returns draws consumed, or -1 if the stream ran
 * out. */
long po_run_stream(po_ctx* c, int n, const uint32_t* stream, long n_stream,
                   int* move_type, int* accept, double* etot);

void po_coords(const po_ctx* c, double* out);
void po_set_coords(po_ctx* c, const double* xyz);
/* {Rg^2, Rgx^2, Rgy^2, Rgz^2, end-to-end^2} */
void po_observables(const po_ctx* c, double* out);
/* One CalcRhoZ pass into out[3*n_bin]; returns n_bin. */
int po_rhoz(const po_ctx* c, double* out, int cap);
/* ForceField::BeadsEnergy (cbmc.cc:5-151) for trial bead b1 and, for a
 * charged species, trial counterion b2 (may be NULL), with cl grown beads
 * chain[cl*3] (and counterions chain_ci); delete_id = -1 for insertion. */
double po_beads_energy(po_ctx* c, const double* b1, const double* b2, int cl,
                       const double* chain, const double* chain_ci, int delete_id);
/* ForceField::CalcPressureForceLJELSlit (pressure.cc:404-488) on the current
 * configuration: out12 = p_tensor[0..11] after this evaluation (6-11 the
 * accumulators: LJ ion, polymer, wall-wall; Ewald ion, polymer, wall-wall). */
void po_pressure_force_slit(po_ctx* c, double* out12);
/* Its inputs: scal = {box[3], ebox[3], npbc, phantom, use_pair, use_ewald,
 * use_ext, pair_kind, ext_kind, lj_cut, lB, alpha, real_cut, real_cell[3],
 * evol, wall_cut, n_type, n_k, n_bead, n_mol} (26 values); per_type[5 n_type] =
 * {lj sigma, lj epsilon, wall sigma, wall epsilon, graft} per type; type,
 * q [n_bead]; mol_start [n_mol + 1]; kv [3 n_k], kw [n_k]. NULL skips one. */
void po_slit_inputs(const po_ctx* c, double* scal, double* per_type, int* type, double* q,
                    int* mol_start, double* kv, double* kw);
/* First n outputs of an mt19937 seeded with `seed`. */
void po_mt19937(uint32_t seed, long n, uint32_t* out);

#ifdef __cplusplus
}
#endif
#endif
