// Harness-side control of the shim runtime (test infrastructure for the oracle).
#ifndef DK_SHIM_HPP
#define DK_SHIM_HPP
namespace dkshim {
// Create the shared control block for `npes` PEs; call once before forking.
int setup(int npes, const char* scratch_dir);
// Set this process's PE number; call in each forked child.
void set_pe(int pe);
}
#endif
