/* Minimal OpenSHMEM surface for compiling DAKC's counting sources on one host
 * (test infrastructure for the oracle; never part of the engine).  PEs are
 * forked processes; see dk_shim.hpp. */
#ifndef DK_SHIM_SHMEM_H
#define DK_SHIM_SHMEM_H
#ifdef __cplusplus
extern "C" {
#endif
int shmem_my_pe(void);
int shmem_n_pes(void);
void shmem_barrier_all(void);
void shmem_init(void);
void shmem_finalize(void);
#ifdef __cplusplus
}
#endif
#endif
