// plum_gpu -- command-line driver with the reference's usage:
//     plum_gpu [seed] [fp32] < run.in
// Reads run.in from stdin (coordinate/topology files relative to the working
// directory), runs the steps of run.in on the GPU through the reference-named
// host classes, writes the reference's output files (stat, trajectories,
// last coordinates, topology and rho(z)) into the working directory, and
// prints the averaged energies, the mean Rg^2 and the acceptance ratio. The reference seeds from the clock (simulation.cc:133-136);
// this driver takes the seed as its first argument (default 5489).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../../../include/plum_host.hpp"

int main(int argc, char** argv) {
  unsigned seed = argc > 1 ? (unsigned)std::strtoul(argv[1], nullptr, 10) : 5489u;
  int form = (argc > 2 && !std::strcmp(argv[2], "fp32")) ? PLUM_FORM_FP32 : PLUM_FORM_FP64;
  try {
    plum::Simulation sim(std::cin, ".", seed, form);
    sim.EnableOutput(".");  // the reference's files in the working directory
    sim.Run();
    sim.Finish();
    const double n = sim.ff_avg_counter > 0 ? (double)sim.ff_avg_counter : 1.0;
    std::printf("steps %ld\n", sim.step);
    std::printf("<PairEne> %.10g <EwaldEne> %.10g <BondEne> %.10g <ExtPotEne> %.10g\n",
                sim.pair_e_cumu / n, sim.ewald_e_cumu / n, sim.bond_e_cumu / n,
                sim.ext_e_cumu / n);
    std::printf("<Rg^2> %.10g\n", sim.mol_avg_counter ? sim.rg_tot_cumu / sim.mol_avg_counter : 0.0);
    std::printf("E_total_now %.12g\n",
                sim.force_field.TotPairEnergy() + sim.force_field.TotEwaldEnergy() +
                    (sim.force_field.UseBondPot() ? sim.force_field.TotBondEnergy() : 0.0) +
                    (sim.force_field.UseExtPot() ? sim.force_field.TotExtEnergy() : 0.0));
  } catch (const std::exception& e) {
    std::fprintf(stderr, "plum_gpu: %s\n", e.what());
    return 1;
  }
  return 0;
}
