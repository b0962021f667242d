// The binding a maintainer of the reference adds to src/solver.cpp, compiled
// against the reference's own headers (compile only, no link): the GPU solve
// template instantiated with lightfem::Model and lightfem::AnalysisResult, so
// every member it reads or writes exists in the reference's types with the
// meaning it assumes.
//
// The one piece the reference has to add is assign_stiffness for its CsrMatrix
// (declared here, defined beside CsrMatrix in src/sparse.cpp, where the private
// arrays are in reach): the retained stiffness comes back as CSR arrays.
#include "lightfem/model.hpp"
#include "lightfem/solver.hpp"
#include "lightfem/sparse.hpp"
#include "lightfem_gpu_solve.hpp"

namespace lightfem {

void assign_stiffness(CsrMatrix& matrix, std::size_t rows, const std::vector<int64_t>& row_offsets,
                      const std::vector<int32_t>& columns, std::vector<double>&& values);

// The `solver gpu` / `solver gpu_mixed` branch of LinearElasticSolver::solve
// (src/solver.cpp:875).
AnalysisResult solve_on_gpu(Model& model) {
    AnalysisResult result;
    lightfem_gpu::solve(model, result, 0);
    return result;
}

}  // namespace lightfem
