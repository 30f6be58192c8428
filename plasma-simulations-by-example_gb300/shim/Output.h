/*
 * Output.h (drop-in) -- the reference's Output namespace
 * (ch3/ver2/Output.h:8-12): VTK ImageData fields, screen line, and the
 * runtime_diags.csv columns, computed on the GPU and read back per call.
 */
#ifndef ESPIC_SHIM_OUTPUT_H
#define ESPIC_SHIM_OUTPUT_H

#include <fstream>
#include <vector>

#include "Species.h"
#include "World.h"

namespace Output {
void fields(World &world, std::vector<Species> &species);
void screenOutput(World &world, std::vector<Species> &species);
void diagOutput(World &world, std::vector<Species> &species);
/* ch4/Output.cpp:175-228: about num_parts particles per species as VTK
 * PolyData (positions, velocities) */
void particles(World &world, std::vector<Species> &species, int num_parts);
}  // namespace Output

#endif
