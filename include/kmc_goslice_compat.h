/*
 * kmc_goslice_compat.h -- the Go library's exported names and signatures,
 * served by the GPU engine.
 *
 * The reference's Python side loads goSimulation/libSimulation.so with ctypes
 * and calls these exports with GoSlice {data, len, cap} views of FP64 arrays
 * (goSimulation/pythonBind.py:28-92, goSimulation/parrallelSimulationBind.py:
 * 50-66).  libkmc_dn_gb300.so exports the same names with the same argument
 * lists, so pointing that path at it (a symlink) runs the reference's own
 * bridge on the GPU engine unchanged.  Semantics follow the Go functions:
 * the single-chain calls start from an empty occupation and write
 * electrode_occupation (and, with record, net traffic and pre-hop
 * occupancy time) into the caller's slices; the return value is the
 * simulated time, or a negative KMC_ERR_* code if the call could not run.
 */
#ifndef KMC_GOSLICE_COMPAT_H
#define KMC_GOSLICE_COMPAT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double *data;
    int64_t len;
    int64_t cap;
} GoSlice;

/* goSimulation/simulationWrapper.go:83-96 */
double wrapperSimulate(int64_t NSites, int64_t NElectrodes, double nu, double kT, double I_0,
                       double R, GoSlice occupation, GoSlice distances, GoSlice E_constant,
                       GoSlice transitions_constant, GoSlice electrode_occupation,
                       GoSlice site_energies, int hops, uint8_t record, GoSlice traffic,
                       GoSlice average_occupation);

/* goSimulation/simulationWrapper.go:128-147 (the default of kmc_dn.go_simulation;
 * its per-state rate cache is not needed: every state is recomputed) */
double wrapperSimulateRecord(int64_t NSites, int64_t NElectrodes, double nu, double kT, double I_0,
                             double R, GoSlice occupation, GoSlice distances, GoSlice E_constant,
                             GoSlice transitions_constant, GoSlice electrode_occupation,
                             GoSlice site_energies, int hops, uint8_t record, GoSlice traffic,
                             GoSlice average_occupation);

/* goSimulation/simulationWrapper.go:149-170 (no record, as in Go) */
double wrapperSimulateRecordPlus(int64_t NSites, int64_t NElectrodes, double nu, double kT,
                                 double I_0, double R, GoSlice occupation, GoSlice distances,
                                 GoSlice E_constant, GoSlice transitions_constant,
                                 GoSlice electrode_occupation, GoSlice site_energies, int hops,
                                 uint8_t record, GoSlice traffic, GoSlice average_occupation);

/* goSimulation/simulationWrapper.go:98-110: pairs with tc <= threshold*max(tc) left out */
double wrapperSimulatePruned(int64_t NSites, int64_t NElectrodes, double prune_threshold, double nu,
                             double kT, double I_0, double R, GoSlice occupation, GoSlice distances,
                             GoSlice E_constant, GoSlice transitions_constant,
                             GoSlice electrode_occupation, GoSlice site_energies, int hops,
                             uint8_t record, GoSlice traffic, GoSlice average_occupation);

/* goSimulation/simulationWrapper.go:224-235: mean-field relaxation
 * (probSimulate, probabilitySimulation.go:53-157) from occupation 0.5 on
 * every acceptor.  Writes occupation (the final probabilities),
 * electrode_occupation (integrated net expected charge), site_energies
 * (acceptor entries) and, with record, traffic / average_occupation
 * (accumulated, as the Go function does).  FP64 arithmetic.  Returns the
 * simulated time, or a negative KMC_ERR_* code. */
double wrapperSimulateProbability(int64_t NSites, int64_t NElectrodes, double nu, double kT,
                                  double I_0, double R, GoSlice occupation, GoSlice distances,
                                  GoSlice E_constant, GoSlice transitions_constant,
                                  GoSlice electrode_occupation, GoSlice site_energies, int hops,
                                  uint8_t record, GoSlice traffic, GoSlice average_occupation);

/* goSimulation/simulationWrapper.go:274-315: ragged batch, one chain per entry,
 * each starting from its own occupation; writes electrode_occupation and time. */
int64_t parallelSimulations(GoSlice NSites, GoSlice NElectrodes, GoSlice nu, GoSlice kT,
                            GoSlice I_0, GoSlice R, GoSlice occupation, GoSlice distances,
                            GoSlice E_constant, GoSlice transitions_constant,
                            GoSlice electrode_occupation, GoSlice hops, GoSlice time,
                            GoSlice site_energies);

/* Returns sum_k (k+1) * s_k.len over fourteen slices, touching nothing else:
 * lets a caller check that its FFI passes fourteen GoSlice arguments the way
 * the platform's C ABI does before it calls parallelSimulations.  No
 * reference counterpart (diagnostic). */
int64_t kmc_goslice_abi_probe(GoSlice s0, GoSlice s1, GoSlice s2, GoSlice s3, GoSlice s4,
                              GoSlice s5, GoSlice s6, GoSlice s7, GoSlice s8, GoSlice s9,
                              GoSlice s10, GoSlice s11, GoSlice s12, GoSlice s13);

#ifdef __cplusplus
}
#endif

#endif /* KMC_GOSLICE_COMPAT_H */
