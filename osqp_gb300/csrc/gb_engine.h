// gb_engine.h -- what the polish stage (polish.cu) reads from a single-QP
// solver's device workspace (engine.cu).
#pragma once

#include <cuda_runtime.h>

#include "osqp_gb300.h"
#include "gb_solver.cuh"

struct GbEngineView {
  gb::DevProblem<OSQPFloat> pr;   // scaled problem and iterates on the device
  gb::DevSettings ds;
  int n, m, nnzA, nnzPf;
  int use_grid, grid_blocks;
  gb::GridSync gs;                // grid barrier buffers (free after the solve)
  cudaStream_t stream;
  gb::SolverScalars* h_st;        // host copy of the solve's scalars
};

GbEngineView gb_engine_view(OSQPSolver* solver);
