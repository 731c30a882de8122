/* Walk through the C API the way an SCF code (and the reference's
 * tests/c_api_test.cxx) uses it: status handling, handle lifetimes, the
 * factories, error strings of the preconditions, and -- with argument "gpu"
 * -- SSF weights and eval_exc_vxc / eval_exc / integrate_den on the device.
 * The system is one water (the reference test's geometry, bohr) in this
 * project's even-tempered basis with PBE; the density is P = C C^T from a
 * fixed linear congruential sequence.  In "gpu" mode the program writes nbf,
 * P, VXC, EXC, EXC-only and N_el to the file named by the second argument
 * for the test to compare with the oracle. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gauxc_gb300.h"

#define OK(st)                                                                  \
  do {                                                                          \
    if ((st).code != 0) {                                                       \
      fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__,                        \
              (st).message ? (st).message : "?");                               \
      return 1;                                                                 \
    }                                                                           \
  } while (0)
#define EXPECT(c)                                                               \
  do {                                                                          \
    if (!(c)) {                                                                 \
      fprintf(stderr, "%s:%d: expectation failed: %s\n", __FILE__, __LINE__, #c); \
      return 1;                                                                 \
    }                                                                           \
  } while (0)
#define FAILS_WITH(st, text)                                                    \
  do {                                                                          \
    EXPECT((st).code != 0 && (st).message && strstr((st).message, text));       \
    gauxc_status_delete(&(st));                                                 \
  } while (0)

static int add_shells(GauXCShell* out, int n, int Z, const double* o) {
  /* O: 10 s (0.08 3^k), 6 p (0.1 3^k), 2 d (0.5 3^k); H: 5 s, 2 p */
  const int nl[2][3] = {{5, 2, 0}, {10, 6, 2}};
  const double a0[3] = {0.08, 0.1, 0.5};
  const int row = Z == 8;
  for (int l = 0; l < 3; ++l)
    for (int k = 0; k < nl[row][l]; ++k) {
      GauXCShell* s = &out[n++];
      memset(s, 0, sizeof(*s));
      s->l = l;
      s->pure = true;
      s->nprim = 1;
      s->exponents[0] = a0[l] * pow(3.0, k);
      s->coefficients[0] = 1.0;
      memcpy(s->origin, o, sizeof(double) * 3);
      s->shell_tolerance = 1e-10;
    }
  return n;
}

int main(int argc, char** argv) {
  const int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
  GauXCStatus st = {0, NULL};

  /* a call clears a prior message; deleting a null status is allowed */
  st.code = 99;
  st.message = (char*)malloc(6);
  memcpy(st.message, "error", 6);
  GauXCMolecule m0 = gauxc_molecule_new(&st);
  EXPECT(st.code == 0 && st.message == NULL);
  gauxc_molecule_delete(&st, &m0);
  EXPECT(m0.ptr == NULL);
  gauxc_status_delete(NULL);

  /* invalid handles */
  GauXCMolecule bad = {{GauXC_Type_Molecule}, NULL};
  EXPECT(gauxc_molecule_natoms(&st, bad) == 0);
  FAILS_WITH(st, "Invalid Molecule handle");

  const GauXCAtom atoms[3] = {{1, 0.0, 1.579252144093028, 2.174611055780858},
                              {8, 0.0, 0.0, 0.0},
                              {1, 0.0, 1.579252144093028, -2.174611055780858}};
  GauXCMolecule mol = gauxc_molecule_new_from_atoms(&st, atoms, 3);
  OK(st);
  EXPECT(gauxc_molecule_natoms(&st, mol) == 3);

  GauXCShell shells[64];
  int nsh = 0;
  for (int i = 0; i < 3; ++i) {
    const double o[3] = {atoms[i].x, atoms[i].y, atoms[i].z};
    nsh = add_shells(shells, nsh, (int)atoms[i].Z, o);
  }
  GauXCBasisSet basis = gauxc_basisset_new_from_shells(&st, shells, (size_t)nsh, true);
  OK(st);
  const int64_t nbf = gauxc_gb300_basisset_nbf(&st, basis);
  OK(st);
  EXPECT(nbf == 60);

  GauXCMolGrid mg = gauxc_molgrid_new_default(&st, mol, GauXC_PruningScheme_Unpruned, 512,
                                              GauXC_RadialQuad_MuraKnowles,
                                              GauXC_AtomicGridSizeDefault_FineGrid);
  OK(st);
  GauXCRuntimeEnvironment rt = gpu ? gauxc_device_runtime_environment_new(&st, 0.5)
                                   : gauxc_runtime_environment_new(&st);
  OK(st);
  EXPECT(gauxc_runtime_environment_comm_rank(&st, rt) == 0);
  EXPECT(gauxc_runtime_environment_comm_size(&st, rt) == 1);

  GauXCLoadBalancerFactory lbf = gauxc_load_balancer_factory_new(&st, GauXC_ExecutionSpace_Host,
                                                                 NULL);
  FAILS_WITH(st, "Load balancer kernel name string cannot be null");
  lbf = gauxc_load_balancer_factory_new(
      &st, gpu ? GauXC_ExecutionSpace_Device : GauXC_ExecutionSpace_Host, "Default");
  OK(st);
  GauXCLoadBalancer lb = gauxc_load_balancer_factory_get_instance(&st, lbf, rt, mol, mg, basis);
  OK(st);
  const size_t ntasks = gauxc_gb300_load_balancer_ntasks(&st, lb);
  EXPECT(ntasks > 0 && !gauxc_gb300_load_balancer_weights_modified(&st, lb));

  GauXCMolecularWeightsSettings ws = {GauXC_XCWeightAlg_Becke, false};
  GauXCMolecularWeightsFactory mwf =
      gauxc_molecular_weights_factory_new(&st, GauXC_ExecutionSpace_Device, "Default", ws);
  FAILS_WITH(st, "Only SSF Supported On Device");
  ws.weight_alg = GauXC_XCWeightAlg_SSF;
  mwf = gauxc_molecular_weights_factory_new(&st, GauXC_ExecutionSpace_Device, "Default", ws);
  OK(st);
  GauXCMolecularWeights mw = gauxc_molecular_weights_factory_get_instance(&st, mwf);
  OK(st);

  GauXCFunctional func = gauxc_functional_from_enum(&st, GauXC_Functional_PBE, false);
  OK(st);
  GauXCIntegrator integ = gauxc_integrator_new(&st, func, lb, GauXC_ExecutionSpace_Device, NULL,
                                               "Default", "Default", "Default");
  FAILS_WITH(st, "Integrator input type string cannot be null");
  integ = gauxc_integrator_new(&st, func, lb, GauXC_ExecutionSpace_Device, "Replicated",
                               "Default", NULL, "Default");
  FAILS_WITH(st, "Local work kernel name string cannot be null");
  integ = gauxc_integrator_new(&st, func, lb, GauXC_ExecutionSpace_Device, "Replicated",
                               "Default", "Default", "Default");
  OK(st);

  /* density P = C C^T, C[nbf x 5] from a linear congruential sequence */
  double* C = (double*)malloc(sizeof(double) * nbf * 5);
  double* P = (double*)malloc(sizeof(double) * nbf * nbf);
  double* V = (double*)malloc(sizeof(double) * nbf * nbf);
  uint64_t x = 12345;
  for (int64_t i = 0; i < nbf * 5; ++i) {
    x = x * 6364136223846793005ULL + 1442695040888963407ULL;
    C[i] = ((double)(x >> 11) / 9007199254740992.0 - 0.5) / sqrt((double)nbf);
  }
  for (int64_t j = 0; j < nbf; ++j)
    for (int64_t i = 0; i < nbf; ++i) {
      double s = 0.;
      for (int k = 0; k < 5; ++k) s += C[i + k * nbf] * C[j + k * nbf];
      P[i + j * nbf] = s;
    }
  double exc = 0., exc_only = 0., den = 0.;
  gauxc_integrator_eval_exc_vxc_rks(&st, integ, nbf, nbf, P, nbf, &exc, V, nbf);
  FAILS_WITH(st, "Weights Have Not Been Modified");
  gauxc_integrator_eval_exc_vxc_rks(&st, integ, nbf, nbf - 1, P, nbf, &exc, V, nbf);
  FAILS_WITH(st, "P Must Be Square");
  gauxc_integrator_eval_exc_vxc_rks(&st, integ, nbf, nbf, NULL, nbf, &exc, V, nbf);
  FAILS_WITH(st, "Density matrix pointer cannot be null");

  if (gpu) {
    gauxc_molecular_weights_modify_weights(&st, mw, lb);
    OK(st);
    EXPECT(gauxc_gb300_load_balancer_weights_modified(&st, lb));
    gauxc_integrator_eval_exc_vxc_rks(&st, integ, nbf, nbf, P, nbf, &exc, V, nbf);
    OK(st);
    gauxc_integrator_eval_exc_rks(&st, integ, nbf, nbf, P, nbf, &exc_only);
    OK(st);
    gauxc_integrator_integrate_den(&st, integ, nbf, nbf, P, nbf, &den);
    OK(st);
    EXPECT(fabs(exc_only - exc) <= 1e-12);
    if (argc > 2) {
      FILE* f = fopen(argv[2], "wb");
      EXPECT(f != NULL);
      fwrite(&nbf, sizeof(int64_t), 1, f);
      fwrite(P, sizeof(double), (size_t)(nbf * nbf), f);
      fwrite(V, sizeof(double), (size_t)(nbf * nbf), f);
      fwrite(&exc, sizeof(double), 1, f);
      fwrite(&exc_only, sizeof(double), 1, f);
      fwrite(&den, sizeof(double), 1, f);
      fclose(f);
    }
    printf("EXC %.15f N_el %.15f\n", exc, den);
  }

  /* release: the generic deleter and the typed ones */
  gauxc_integrator_delete(&st, &integ);
  void* obj = &func; /* the generic deleter takes the handle's address */
  gauxc_object_delete(&st, &obj);
  OK(st);
  obj = &mw;
  gauxc_object_delete(&st, &obj);
  OK(st);
  EXPECT(func.ptr == NULL && mw.ptr == NULL);
  gauxc_molecular_weights_factory_delete(&st, &mwf);
  gauxc_load_balancer_delete(&st, &lb);
  gauxc_load_balancer_factory_delete(&st, &lbf);
  gauxc_runtime_environment_delete(&st, &rt);
  gauxc_molgrid_delete(&st, &mg);
  gauxc_basisset_delete(&st, &basis);
  gauxc_molecule_delete(&st, &mol);
  OK(st);
  EXPECT(integ.ptr == NULL && lb.ptr == NULL && mol.ptr == NULL);
  free(C);
  free(P);
  free(V);
  printf("%s walk ok\n", gpu ? "device" : "host");
  return 0;
}
