/*
 * so_entry.c — running the library as a program prints its options.
 *
 * The reference links its library with an entry point and a program
 * interpreter (entry.c:4-11, meson.build:25: -eentry), so that executing
 * libblas2cuda.so prints the BLAS2CUDA_OPTIONS help and exits.  The same
 * holds here for libgbxblas.so and libgbxblas_preload.so (the latter also
 * prints the OBJTRACKER_OPTIONS help).  Loading the library with LD_PRELOAD
 * or dlopen ignores both: the interpreter path is only read when the file is
 * executed, and the entry point is never called.
 */
#include <unistd.h>

#if defined(__x86_64__)
const char gbx_program_interpreter[] __attribute__((section(".interp"))) = "/lib64/ld-linux-x86-64.so.2";
#define GBX_ENTRY_ATTR __attribute__((used, noreturn, force_align_arg_pointer))
#elif defined(__aarch64__)
const char gbx_program_interpreter[] __attribute__((section(".interp"))) = "/lib/ld-linux-aarch64.so.1";
#define GBX_ENTRY_ATTR __attribute__((used, noreturn))
#else
#error "unsupported host architecture for the program entry point"
#endif

void gbx_print_options(int fd);
void gbx_tracker_print_options(void) __attribute__((weak));

/* Entered directly from the dynamic loader (no C runtime start-up frame, the
 * stack as the kernel left it): only write(2) and _exit(2). */
GBX_ENTRY_ATTR void gbx_so_entry(void)
{
    gbx_print_options(STDOUT_FILENO);
    if (gbx_tracker_print_options) gbx_tracker_print_options();
    _exit(0);
}
