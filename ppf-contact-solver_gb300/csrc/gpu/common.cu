// common.cu -- CUDA error handling and the fatal-report state of the ABI.
#include "common.cuh"
#include "fatal.cuh"

#include <stdexcept>
#include <string>

// Fatal code and one-line detail read by the driver's atexit hook
// (crates/ppf-cts-solver/src/cpp/main/main.cu:1656-1668).
extern "C" {
unsigned char g_ppf_fatal_code = 0;
char g_ppf_fatal_detail[512] = {0};
}

namespace ppf {

void set_fatal(unsigned char code, const char *detail) {
    g_ppf_fatal_code = code;
    snprintf(g_ppf_fatal_detail, sizeof(g_ppf_fatal_detail), "%s", detail);
    if (char *nl = strchr(g_ppf_fatal_detail, '\n')) *nl = '\0';
}

namespace gpu {

std::atomic<unsigned long long> g_kernel_launches{0};
thread_local unsigned long long t_kernel_launches = 0;
std::atomic<unsigned long long> g_h2d_bytes{0}, g_d2h_bytes{0};
std::atomic<unsigned long long> g_buffer_epoch{0};
thread_local bool g_capturing = false;

void buffer_grow_during_capture() {
    throw FatalError(4, "a device buffer had to grow while a Newton iteration was being captured");
}

void check_cuda(cudaError_t err, const char *what, const char *file, int line) {
    if (err == cudaSuccess) return;
    char buf[512];
    snprintf(buf, sizeof(buf), "CUDA error %s (%s) at %s:%d in %s",
             cudaGetErrorName(err), cudaGetErrorString(err), file, line, what);
    unsigned char code = err == cudaErrorMemoryAllocation
                             ? 2 /* PPF_FATAL_OOM */
                             : 3 /* PPF_FATAL_CUDA_DRIVER */;
    throw FatalError(code, buf);
}

} // namespace gpu
} // namespace ppf

// Logging sink. The reference driver binary defines print_rust
// (crates/ppf-cts-solver/src/main.rs:48); a strong definition there takes
// precedence over this weak one, which prints to stdout when the library is
// loaded by any other host.
extern "C" __attribute__((weak)) void print_rust(const char *message) {
    fputs(message, stdout);
    fputc('\n', stdout);
}
