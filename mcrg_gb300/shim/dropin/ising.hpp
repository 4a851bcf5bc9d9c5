// ising.hpp -- drop-in for kim-jane/MCRG src/ising.hpp: IsingModel over the
// GPU (declared with Lattice in ../mcrg_classes.hpp).
#pragma once
#include <memory>

#include "lattice.hpp"
