/*
 * GPUScaffoldSimulation.h -- the names the reference's own driver takes from
 * its header of this name, on top of scaffold_compat.h.
 *
 * The reference's driver (SimulationModule/Scaffold/main.cu) includes
 * "GPUScaffoldSimulation.h" and uses, besides the six calls that
 * scaffold_compat.h declares: DEV_NUM (GPUScaffoldSimulation.h:37), sec and
 * T_MAX (option.h:4,6), INPUT_STIM_NUM (UserInputFunctions.h:21), the
 * enumeration counts TotalNumOfCellTypes, TotalNumOfConnectivityTypes and
 * NumOfPlasticity (struct_enum_def.h:10-53), and
 * Env.Host_sim_val[0].Host.neuron_num (struct_enum_def.h:132-171).  With this
 * directory on the include path ahead of the reference's own, that file
 * compiles unchanged and links against libscaffold_gb300.so.  The values are
 * the reference's; they are an interface, not an implementation.
 */
#ifndef SGB_COMPAT_GPU_SCAFFOLD_SIMULATION_H
#define SGB_COMPAT_GPU_SCAFFOLD_SIMULATION_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "../scaffold_compat.h"

#define DEV_NUM 1                 /* one GPU                                   */
#define sec (1000.)               /* ms per second                             */
#define DT (0.1)                  /* substep, ms                               */
#define T_MAX (1000)              /* ms of one trial                           */
#define STEP_MAX ((int)(1 / DT))  /* substeps per 1-ms exchange step           */
#define INPUT_STIM_NUM 2          /* stimulus lists: background, tone          */

/* Cell and projection types of the reference scaffold, in its order. */
enum NeuronType {
  NONE = -1,
  granule_cell,
  glomerulus,
  purkinje_cell,
  golgi_cell,
  stellate_cell,
  basket_cell,
  dcn_cell,
  TotalNumOfCellTypes
};

enum ConnectionType {
  C_NONE = -1,
  parallel_fiber_to_purkinje,
  parallel_fiber_to_golgi,
  parallel_fiber_to_stellate,
  parallel_fiber_to_basket,
  aa_to_golgi,
  aa_to_purkinje,
  golgi_to_golgi,
  stellate_to_stellate,
  basket_to_basket,
  glomerulus_to_dcn,
  purkinje_to_dcn,
  basket_to_purkinje,
  stellate_to_purkinje,
  glomerulus_to_granule,
  glomerulus_to_golgi,
  golgi_to_granule,
  TotalNumOfConnectivityTypes
};

enum DeviceType { NORMAL, INPUT, OUTPUT };

/* No plasticity is switched on in the reference scaffold. */
enum PLASTICITY_LOCATION { NumOfPlasticity };

#endif /* SGB_COMPAT_GPU_SCAFFOLD_SIMULATION_H */
