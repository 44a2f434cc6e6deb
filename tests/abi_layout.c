/* Layout and load check of the C-ABI from C (compiled by tests/test_abi_layout.py with gcc).
 *
 *   abi_layout layout        print "name offset size" for every member of the two structs, in order
 *   abi_layout create LIB    dlopen LIB, call dftbgpu_create on device 0 and print its status (and
 *                            destroy the context when one was created)
 */
#include <dlfcn.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include "dftbgpu.h"

#define FIELD(T, f) printf(#T " " #f " %zu %zu\n", offsetof(T, f), sizeof(((T *)0)->f))

int main(int argc, char **argv) {
  if (argc >= 2 && strcmp(argv[1], "layout") == 0) {
    printf("dftbgpu_scc_opts sizeof %zu\n", sizeof(dftbgpu_scc_opts));
    FIELD(dftbgpu_scc_opts, kT);
    FIELD(dftbgpu_scc_opts, scc_tol);
    FIELD(dftbgpu_scc_opts, max_iter);
    FIELD(dftbgpu_scc_opts, min_iter);
    FIELD(dftbgpu_scc_opts, mix_alpha);
    FIELD(dftbgpu_scc_opts, mix_omega0);
    FIELD(dftbgpu_scc_opts, mix_min_weight);
    FIELD(dftbgpu_scc_opts, mix_max_weight);
    FIELD(dftbgpu_scc_opts, mix_weight_fac);
    FIELD(dftbgpu_scc_opts, net_charge);
    FIELD(dftbgpu_scc_opts, precision);
    FIELD(dftbgpu_scc_opts, convergent_only);
    FIELD(dftbgpu_scc_opts, mixed_switch_tol);
    printf("dftbgpu_energies sizeof %zu\n", sizeof(dftbgpu_energies));
    FIELD(dftbgpu_energies, EnonSCC);
    FIELD(dftbgpu_energies, Escc);
    FIELD(dftbgpu_energies, Erep);
    FIELD(dftbgpu_energies, Eband);
    FIELD(dftbgpu_energies, TS);
    FIELD(dftbgpu_energies, E0);
    FIELD(dftbgpu_energies, Etotal);
    FIELD(dftbgpu_energies, EMermin);
    return 0;
  }
  if (argc >= 3 && strcmp(argv[1], "create") == 0) {
    void *h = dlopen(argv[2], RTLD_NOW | RTLD_LOCAL);
    if (!h) {
      printf("dlopen failed: %s\n", dlerror());
      return 2;
    }
    typedef int (*create_t)(dftbgpu_ctx **, int);
    typedef int (*destroy_t)(dftbgpu_ctx *);
    create_t create = (create_t)dlsym(h, "dftbgpu_create");
    destroy_t destroy = (destroy_t)dlsym(h, "dftbgpu_destroy");
    if (!create || !destroy) {
      printf("missing symbol\n");
      return 3;
    }
    dftbgpu_ctx *ctx = NULL;
    int rc = create(&ctx, 0);
    printf("create %d\n", rc);
    if (rc == DFTBGPU_OK) destroy(ctx);
    return 0;
  }
  fprintf(stderr, "usage: abi_layout layout | create LIB\n");
  return 1;
}
