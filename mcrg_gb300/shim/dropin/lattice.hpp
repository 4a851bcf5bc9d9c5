// lattice.hpp -- drop-in for kim-jane/MCRG src/lattice.hpp.
//
// With this directory first on the quote-include path (and the reference's
// src/ after it, for definitions.hpp, rgnn.hpp and Eigen), the reference's
// own call sites -- src/main.cpp, src/train.cpp, src/rgnn.cpp -- compile
// unchanged against the GPU classes of ../mcrg_classes.hpp: Lattice,
// IsingModel and MonteCarloRenormalizationGroup with the reference's
// members, spins_ an Eigen `imat` host mirror of the device lattice.
#pragma once
#include <mpi.h>

#include "definitions.hpp"
#ifndef MCRG_EIGEN_SPINS
#define MCRG_EIGEN_SPINS 1
#endif
#include "mcrg_classes.hpp"  // found through -I mcrg_gb300/shim
