// C-linkage entry into the reference FWI driver `cufd` (deps/CustomOps/FWI/Src/libCUFD.cu:34-38)
// when the reference sources are compiled for the host CPU through cuda_host_shim.h.
// TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py and by the oracle
// cross-check tests to pin oracle/fwi_oracle.cpp against the reference itself.
#include <string>

void cufd(double* misfit, double* grad_Lambda, double* grad_Mu, double* grad_Den, double* grad_stf,
          const double* Lambda, const double* Mu, const double* Den, const double* stf, int calc_id,
          const int gpu_id, int group_size, const int* shot_ids, const std::string para_fname);

extern "C" int refhost_cufd(double* misfit, double* grad_lambda, double* grad_mu, double* grad_den,
                            double* grad_stf, const double* lambda, const double* mu, const double* den,
                            const double* stf, int calc_id, int group_size, const int* shot_ids,
                            const char* para_fname) {
  cufd(misfit, grad_lambda, grad_mu, grad_den, grad_stf, lambda, mu, den, stf, calc_id, 0, group_size, shot_ids,
       std::string(para_fname));
  return 0;
}
