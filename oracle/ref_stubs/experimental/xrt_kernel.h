// No-op stand-ins for the few XRT host-API types and calls the reference
// host names (GraphDriver.h/.cpp, the device set-up in Placer::Placer), so that
// its CPU path compiles on a machine without XRT.  TEST INFRASTRUCTURE ONLY:
// the harness (oracle/ref_placer.cpp) runs the placer with use_aie false, so
// none of these is ever called.
#pragma once
#include <cstddef>
#include <string>
typedef int xrtMemoryGroup;
enum xclBOSyncDirection { XCL_BO_SYNC_BO_TO_DEVICE = 0, XCL_BO_SYNC_BO_FROM_DEVICE = 1 };
namespace xrt {
struct uuid {};
struct device {
    device() {}
    explicit device(unsigned int) {}
    uuid load_xclbin(const std::string &) { return uuid(); }
};
struct kernel {
    kernel() {}
    kernel(const device &, const uuid &, const std::string &) {}
    xrtMemoryGroup group_id(int) const { return 0; }
};
struct bo {
    bo() {}
    bo(const device &, std::size_t, xrtMemoryGroup) {}
    template <class T> void write(const T *) {}
    template <class T> void read(T *) {}
    void sync(xclBOSyncDirection) {}
};
struct run {
    run() {}
    explicit run(const kernel &) {}
    template <class T> void set_arg(int, const T &) {}
    void start() {}
    void wait() {}
};
}  // namespace xrt
