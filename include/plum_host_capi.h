/* plum_host_capi.h -- C entry points that drive the C++ host classes of
 * include/plum_host.hpp (the reference's Simulation surface) from C callers:
 * tests, scripting languages, the command-line driver.
 *
 * Each replaces a reference call sequence:
 *   plum_sim_create              Simulation::Simulation (simulation.cc:23-201)
 *                                with an explicit seed (the reference seeds
 *                                from the clock, simulation.cc:133-136)
 *   plum_sim_translational_moves Simulation::TranslationalMove
 *                                (simulation.cc:241-355), host control flow,
 *                                energies on the GPU
 *   plum_sim_run_steps           the step loop of Simulation::Run
 *                                (simulation.cc:216-239) on the GPU
 *   plum_sim_steps               the same loop with host control flow,
 *                                Simulation::GCMove (simulation.cc:357-404)
 *                                included
 *   plum_sim_energies            ForceField::Tot*Energy (force_field.cc:1201-1219)
 */
#ifndef PLUM_HOST_CAPI_H_
#define PLUM_HOST_CAPI_H_

#include "plum_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plum_sim plum_sim;

int plum_sim_create(const char* dir, const char* runin_text, unsigned seed, int form,
                    plum_sim** out);
int plum_sim_destroy(plum_sim* sim);
/* n steps of the host control flow; per step the move type (-1 none) and
 * accept flag (host buffers of n, may be NULL). Each step also takes the
 * draw simulation.cc:221 spends on the grand-canonical check. */
int plum_sim_translational_moves(plum_sim* sim, int n, int* move_type, int* accept);
int plum_sim_run_steps(plum_sim* sim, long n);
/* n steps of Simulation::Run's loop (simulation.cc:219-226) with host
 * control flow, grand-canonical exchanges included: per step the move type
 * (0-4 translational, 5 insertion, 6 deletion attempt, -1 none) and whether
 * it was accepted. */
int plum_sim_steps(plum_sim* sim, int n, int* move_type, int* accept);
/* Beads currently in the host molecules (changes with exchanges). */
int plum_sim_n_bead(plum_sim* sim);
int plum_sim_positions(plum_sim* sim, double* xyz);
int plum_sim_energies(plum_sim* sim, double* out);
/* Simulation::EnableOutput: the reference's output files go into dir
 * (simulation.cc:120-131); then plum_sim_run runs the steps of run.in
 * (Simulation::Run, sampling and writing where the reference does) and
 * plum_sim_finish makes the writes of the reference's destructor and closes
 * the files. */
int plum_sim_enable_output(plum_sim* sim, const char* dir);
/* Simulation::WriteCheckpoint / ReadCheckpoint (exact restart, runs with
 * grand-canonical exchange included). */
int plum_sim_write_checkpoint(plum_sim* sim, const char* path);
int plum_sim_read_checkpoint(plum_sim* sim, const char* path);
int plum_sim_run(plum_sim* sim);
/* ForceField::CalcChemicalPotentialF on the current configuration with the
 * simulation's generator (Widom average of 50 test insertions). */
int plum_sim_chem_pot(plum_sim* sim, double* out);
/* ForceField::p_tensor[0..11] and the number of pressure evaluations so far
 * (out13[12]); with eval != 0 one more evaluation of
 * CalcPressureForceLJELSlit on the current configuration first. */
int plum_sim_pressure(plum_sim* sim, int eval, double* out13);
int plum_sim_finish(plum_sim* sim);

#ifdef __cplusplus
}
#endif
#endif
