/*
 * CL/cl.hpp stand-in -- TEST INFRASTRUCTURE ONLY.
 *
 * Just enough of the OpenCL C++ bindings' names for the reference host class
 * (lbmcl.hpp and libs/CLUtil.hpp) to compile on a machine without OpenCL, so
 * that oracle/ref_writers.cpp can call the reference's own file writers
 * (storeMap / storeF / storeData) on host data.  Nothing here talks to a
 * device: every call succeeds and does nothing, except
 * CommandQueue::enqueueReadBuffer, which copies from the host array a Buffer
 * stands for.  Error codes only need to be distinct; the values are this
 * stub's own.
 */
#pragma once

#include <cstddef>
#include <cstring>
#include <exception>
#include <string>
#include <utility>
#include <vector>

typedef int cl_int;
typedef unsigned int cl_uint;
typedef unsigned int cl_bool;
typedef unsigned long long cl_ulong;
typedef cl_ulong cl_bitfield;
typedef cl_bitfield cl_mem_flags;
typedef cl_bitfield cl_device_type;
typedef cl_bitfield cl_command_queue_properties;

#define CL_TRUE 1u
#define CL_SUCCESS 0
/* distinct negative codes for the error-string switch */
#define CL_DEVICE_NOT_FOUND -1
#define CL_DEVICE_NOT_AVAILABLE -2
#define CL_COMPILER_NOT_AVAILABLE -3
#define CL_MEM_OBJECT_ALLOCATION_FAILURE -4
#define CL_OUT_OF_RESOURCES -5
#define CL_OUT_OF_HOST_MEMORY -6
#define CL_PROFILING_INFO_NOT_AVAILABLE -7
#define CL_MEM_COPY_OVERLAP -8
#define CL_IMAGE_FORMAT_MISMATCH -9
#define CL_IMAGE_FORMAT_NOT_SUPPORTED -10
#define CL_BUILD_PROGRAM_FAILURE -11
#define CL_MAP_FAILURE -12
#define CL_MISALIGNED_SUB_BUFFER_OFFSET -13
#define CL_EXEC_STATUS_ERROR_FOR_EVENTS_IN_WAIT_LIST -14
#define CL_COMPILE_PROGRAM_FAILURE -15
#define CL_LINKER_NOT_AVAILABLE -16
#define CL_LINK_PROGRAM_FAILURE -17
#define CL_DEVICE_PARTITION_FAILED -18
#define CL_KERNEL_ARG_INFO_NOT_AVAILABLE -19
#define CL_INVALID_VALUE -30
#define CL_INVALID_DEVICE_TYPE -31
#define CL_INVALID_PLATFORM -32
#define CL_INVALID_DEVICE -33
#define CL_INVALID_CONTEXT -34
#define CL_INVALID_QUEUE_PROPERTIES -35
#define CL_INVALID_COMMAND_QUEUE -36
#define CL_INVALID_HOST_PTR -37
#define CL_INVALID_MEM_OBJECT -38
#define CL_INVALID_IMAGE_FORMAT_DESCRIPTOR -39
#define CL_INVALID_IMAGE_SIZE -40
#define CL_INVALID_SAMPLER -41
#define CL_INVALID_BINARY -42
#define CL_INVALID_BUILD_OPTIONS -43
#define CL_INVALID_PROGRAM -44
#define CL_INVALID_PROGRAM_EXECUTABLE -45
#define CL_INVALID_KERNEL_NAME -46
#define CL_INVALID_KERNEL_DEFINITION -47
#define CL_INVALID_KERNEL -48
#define CL_INVALID_ARG_INDEX -49
#define CL_INVALID_ARG_VALUE -50
#define CL_INVALID_ARG_SIZE -51
#define CL_INVALID_KERNEL_ARGS -52
#define CL_INVALID_WORK_DIMENSION -53
#define CL_INVALID_WORK_GROUP_SIZE -54
#define CL_INVALID_WORK_ITEM_SIZE -55
#define CL_INVALID_GLOBAL_OFFSET -56
#define CL_INVALID_EVENT_WAIT_LIST -57
#define CL_INVALID_EVENT -58
#define CL_INVALID_OPERATION -59
#define CL_INVALID_GL_OBJECT -60
#define CL_INVALID_BUFFER_SIZE -61
#define CL_INVALID_MIP_LEVEL -62
#define CL_INVALID_GLOBAL_WORK_SIZE -63
#define CL_INVALID_PROPERTY -64
#define CL_INVALID_IMAGE_DESCRIPTOR -65
#define CL_INVALID_COMPILER_OPTIONS -66
#define CL_INVALID_LINKER_OPTIONS -67
#define CL_INVALID_DEVICE_PARTITION_COUNT -68

#define CL_MEM_READ_WRITE (1ull << 0)
#define CL_MEM_HOST_READ_ONLY (1ull << 8)
#define CL_MEM_HOST_NO_ACCESS (1ull << 9)
#define CL_DEVICE_TYPE_CPU (1ull << 1)
#define CL_DEVICE_TYPE_GPU (1ull << 2)
#define CL_QUEUE_PROFILING_ENABLE (1ull << 1)

/* info names: string-valued below 100, integer-valued from 100 */
#define CL_PLATFORM_NAME 1
#define CL_PLATFORM_VENDOR 2
#define CL_PLATFORM_VERSION 3
#define CL_DEVICE_NAME 4
#define CL_DEVICE_VENDOR 5
#define CL_PROGRAM_BUILD_LOG 6
#define CL_DEVICE_TYPE 100
#define CL_DEVICE_MAX_COMPUTE_UNITS 101
#define CL_DEVICE_GLOBAL_MEM_SIZE 102
#define CL_DEVICE_MAX_CLOCK_FREQUENCY 103
#define CL_DEVICE_MAX_MEM_ALLOC_SIZE 104
#define CL_DEVICE_LOCAL_MEM_SIZE 105
#define CL_DEVICE_AVAILABLE 106
#define CL_PROFILING_COMMAND_START 107
#define CL_PROFILING_COMMAND_END 108
#define CL_KERNEL_WORK_GROUP_SIZE 109
#define CL_KERNEL_LOCAL_MEM_SIZE 110
#define CL_KERNEL_PRIVATE_MEM_SIZE 111
#define CL_KERNEL_PREFERRED_WORK_GROUP_SIZE_MULTIPLE 112

namespace cl {

template <int N> struct InfoType { typedef cl_ulong type; };
template <> struct InfoType<CL_PLATFORM_NAME> { typedef std::string type; };
template <> struct InfoType<CL_PLATFORM_VENDOR> { typedef std::string type; };
template <> struct InfoType<CL_PLATFORM_VERSION> { typedef std::string type; };
template <> struct InfoType<CL_DEVICE_NAME> { typedef std::string type; };
template <> struct InfoType<CL_DEVICE_VENDOR> { typedef std::string type; };
template <> struct InfoType<CL_PROGRAM_BUILD_LOG> { typedef std::string type; };

class Error : public std::exception {
    cl_int code_;

  public:
    explicit Error(cl_int code = CL_SUCCESS) : code_(code) {}
    cl_int err() const { return code_; }
    const char *what() const noexcept override { return "stub"; }
};

class NDRange {
    size_t v_[3];

  public:
    NDRange() : v_{0, 0, 0} {}
    explicit NDRange(size_t x) : v_{x, 1, 1} {}
    NDRange(size_t x, size_t y, size_t z) : v_{x, y, z} {}
    size_t operator[](int i) const { return v_[i]; }
};
static const NDRange NullRange;

class Device {
  public:
    template <int N> typename InfoType<N>::type getInfo() const { return typename InfoType<N>::type(); }
};

class Platform {
  public:
    static cl_int get(std::vector<Platform> *p)
    {
        p->assign(1, Platform());
        return CL_SUCCESS;
    }
    template <int N> typename InfoType<N>::type getInfo() const { return typename InfoType<N>::type(); }
    cl_int getDevices(cl_device_type, std::vector<Device> *d) const
    {
        d->assign(1, Device());
        return CL_SUCCESS;
    }
};

class Context {
  public:
    Context() {}
    explicit Context(const Device &) {}
};

/* A Buffer stands for a host array (`host`, set by the test harness). */
class Buffer {
  public:
    const void *host = nullptr;
    Buffer() {}
    Buffer(const Context &, cl_mem_flags, size_t, void *, cl_int *err = nullptr)
    {
        if (err) *err = CL_SUCCESS;
    }
};

class Program {
  public:
    typedef std::vector<std::pair<const char *, size_t>> Sources;
    Program() {}
    Program(const Context &, const Sources &) {}
    cl_int build(const char *) { return CL_SUCCESS; }
    template <int N> std::string getBuildInfo(const Device &) const { return std::string(); }
};

class Kernel {
  public:
    Kernel() {}
    Kernel(const Program &, const char *, cl_int *err = nullptr)
    {
        if (err) *err = CL_SUCCESS;
    }
    template <class A> cl_int setArg(cl_uint, const A &) { return CL_SUCCESS; }
};

class Event {
  public:
    template <int N> cl_ulong getProfilingInfo() const { return 0; }
    cl_int wait() const { return CL_SUCCESS; }
};

class CommandQueue {
  public:
    CommandQueue() {}
    CommandQueue(const Context &, const Device &, cl_command_queue_properties) {}
    cl_int enqueueReadBuffer(const Buffer &b, cl_bool, size_t offset, size_t size, void *ptr,
                             const std::vector<Event> * = nullptr, Event * = nullptr) const
    {
        std::memcpy(ptr, static_cast<const char *>(b.host) + offset, size);
        return CL_SUCCESS;
    }
    cl_int enqueueNDRangeKernel(const Kernel &, const NDRange &, const NDRange &, const NDRange &,
                                const std::vector<Event> * = nullptr, Event * = nullptr) const
    {
        return CL_SUCCESS;
    }
    cl_int finish() const { return CL_SUCCESS; }
};

}  // namespace cl
