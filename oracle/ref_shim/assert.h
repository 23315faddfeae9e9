// Host stand-in for <assert.h> in the reference-side parity harness (TEST
// INFRASTRUCTURE ONLY).  A failed assert in ros_tsdf's device code would stop
// the kernel; here it is counted (ref_assert_failures) and the thread goes on,
// so the harness reports the count instead of aborting the test process.
// Like the system header, this file has no include guard.
#include_next <assert.h>
#undef assert
#ifdef __cplusplus
void ref_assert_failed(const char* expr, const char* file, int line);
#define assert(e) ((e) ? (void)0 : ref_assert_failed(#e, __FILE__, __LINE__))
#endif
