// muesli.h -- runtime of the GB300 skeleton front end (drop-in for the Muesli
// reference's include/muesli.h).
//
// Programs written against the reference include "muesli.h", "da.h", "dm.h"
// and "dc.h", call msl::initSkeletons(argc, argv) first and
// msl::terminateSkeletons() last, and pass functors tagged MSL_USERFUNC to
// the skeletons. Compiled with nvcc for sm_103a and linked against
// libmsl_gb300.so, the same source runs on one GB300: the distributed
// partition collapses to one device-resident partition, there are no MPI
// ranks, and skeletons are enqueued asynchronously on the library stream,
// synchronising only when the host reads data.
//
// Reference: include/muesli.h:86-318 (macros, Muesli statics, setters),
// src/muesli.cpp:63-294 (init/terminate, syncStreams, timing, throws).
#pragma once

#include <cuda_runtime.h>

// The standard headers the reference's muesli.h provides to the programs
// that include it (include/muesli.h:40-58).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "msl_gb300.h"
#include "msl_single_rank_mpi.h"

#define MSL_USERFUNC __host__ __device__
#define MSL_GPUFUNC __device__
#define MSL_CPUFUNC __host__

namespace msl {

enum Distribution { DIST, COPY };

// Global configuration (include/muesli.h:149-181). With one device and one
// process most fields are informational: proc_id is 0, num_total_procs 1, and
// cpu_fraction is accepted but ignored (every element lives on the GPU).
class Muesli {
   public:
    static inline int proc_id = 0;
    static inline int proc_entrance = -1;
    static inline int running_proc_no = 0;
    static inline int num_total_procs = 1;
    static inline int num_local_procs = 1;
    static inline double start_time = 0.0;
    static inline char *program_name = nullptr;
    static inline int distribution_mode = 0;
    static inline int task_group_size = 256;
    static inline int num_conc_kernels = 16;
    static inline int num_threads = 1;
    static inline int num_runs = 1;
    static inline int num_gpus = 1;
    static inline int reps = 1;
    static inline double cpu_fraction = 0.0;
    static inline int max_gpus = 1;
    static inline int threads_per_block = 1024;
    static inline int tpb_x = 16;
    static inline int tpb_y = 16;
    static inline bool debug = false;
    static inline bool use_timer = false;
    static inline int elem_per_thread = 1;
    static inline std::vector<cudaStream_t> streams;
};

static const int ANY_TAG = -1;
static const int MYTAG = 1;
static const int STOPTAG = 2;
static const int UNDEFINED = -1;
static const int DEFAULT_TASK_GOUP_SIZE = 256;
static const int DEFAULT_NUM_CONC_KERNELS = 16;
static const int DEFAULT_NUM_RUNS = 1;
static const int DEFAULT_TILE_WIDTH = 16;

namespace detail {
// Exception vocabulary of include/detail/exception.h. As in the reference,
// throws() prints the message and execution continues.
class Exception {
   public:
    virtual ~Exception() {}
    virtual std::string what() const = 0;
};
#define MSL_DEFINE_EXCEPTION(Name, Text)                         \
    class Name : public Exception {                              \
       public:                                                   \
        std::string what() const override { return Text; }       \
    };
MSL_DEFINE_EXCEPTION(NotYetImplementedException, "NotYetImplementedException")
MSL_DEFINE_EXCEPTION(NotSameSizeException, "NotSameSizeException")
MSL_DEFINE_EXCEPTION(MissingInitializationException, "MissingInitializationException")
MSL_DEFINE_EXCEPTION(IllegalGetException, "IllegalGetException")
MSL_DEFINE_EXCEPTION(IllegalPutException, "IllegalPutException")
MSL_DEFINE_EXCEPTION(IndexOutOfBoundsException, "IndexOutOfBoundsException")
MSL_DEFINE_EXCEPTION(SizeMismatchException, "SizeMismatchException")
MSL_DEFINE_EXCEPTION(DeviceOutOfMemory, "DeviceOutOfMemory")
MSL_DEFINE_EXCEPTION(InvalidCube, "InvalidCube")
MSL_DEFINE_EXCEPTION(FeatureNotSupportedByDeviceException, "FeatureNotSupportedByDeviceException")
MSL_DEFINE_EXCEPTION(InternalErrorException, "InternalErrorException")
MSL_DEFINE_EXCEPTION(IllegalArgumentException, "IllegalArgumentException")
MSL_DEFINE_EXCEPTION(IllegalPartitionException, "IllegalPartitionException")
MSL_DEFINE_EXCEPTION(RotateRowManyNotImplementedException, "RotateRowManyNotImplementedException")
#undef MSL_DEFINE_EXCEPTION
}  // namespace detail

inline void throws(const detail::Exception &e) { std::cout << e.what() << std::endl; }

// Check a libmsl_gb300 status: print-and-continue like the reference's
// throws(), or throw std::runtime_error when MSL_THROW_ON_ERROR is defined.
inline bool check_status(int rc, const char *what) {
    if (rc == MSL_OK) return true;
#ifdef MSL_THROW_ON_ERROR
    throw std::runtime_error(std::string(what) + ": " + msl_last_error_string());
#else
    std::fprintf(stderr, "msl: %s failed (%d): %s\n", what, rc, msl_last_error_string());
    return false;
#endif
}

inline cudaStream_t stream() {
    void *s = nullptr;
    msl_get_stream(&s);
    return (cudaStream_t)s;
}
inline int sm_count() {
    static int sms = 0;
    if (!sms) msl_device_info(&sms, nullptr, nullptr);
    return sms;
}

inline std::chrono::steady_clock::time_point &timer_origin() {
    static std::chrono::steady_clock::time_point t;
    return t;
}
inline double wtime() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// src/muesli.cpp:63-110: bind device 0, create the stream, default settings.
inline void initSkeletons(int argc, char **argv, bool debug = false) {
    if (argc >= 1 && argv) Muesli::program_name = argv[0];
    int dev = 0;
    if (const char *e = std::getenv("MSL_DEVICE")) dev = std::atoi(e);
    check_status(msl_init(dev), "initSkeletons");
    Muesli::proc_entrance = 0;
    Muesli::debug = debug;
    Muesli::num_gpus = 1;
    Muesli::max_gpus = 1;
    Muesli::streams.assign(1, stream());
    Muesli::start_time = wtime();
}
// Release hooks of front-end resources (scratch buffers), run by terminateSkeletons().
inline std::vector<void (*)()> &at_terminate() {
    static std::vector<void (*)()> hooks;
    return hooks;
}

// src/muesli.cpp:112-158.
inline void terminateSkeletons() {
    msl_sync();
    for (auto h : at_terminate()) h();
    at_terminate().clear();
    check_status(msl_terminate(), "terminateSkeletons");
    Muesli::proc_entrance = -1;
    Muesli::streams.clear();
}
// src/muesli.cpp:213-223: wait for the skeletons enqueued so far.
inline void syncStreams() { check_status(msl_sync(), "syncStreams"); }

inline void printv(const char *format, ...) {
    va_list ap;
    va_start(ap, format);
    std::vprintf(format, ap);
    va_end(ap);
}
inline bool isRootProcess() { return Muesli::proc_id == 0; }
inline void setNumThreads(int n) { Muesli::num_threads = n; }
inline void setNumRuns(int n) { Muesli::num_runs = n; }
inline void setNumGpus(int n) { Muesli::num_gpus = n < 1 ? 1 : 1; }
inline void setThreadsPerBlock(int tpb) { Muesli::threads_per_block = tpb; }
inline void setThreadsPerBlock(int x, int y) {
    Muesli::tpb_x = x;
    Muesli::tpb_y = y;
}
inline void setNumConcurrentKernels(int n) { Muesli::num_conc_kernels = n; }
inline void setTaskGroupSize(int n) { Muesli::task_group_size = n; }
inline void setDebug(bool v) { Muesli::debug = v; }
inline void setReps(int v) { Muesli::reps = v; }

// Timing (src/muesli.cpp:248-276): device work is included because every
// split synchronises the library stream first.
inline double &timing_start() {
    static double t = 0.0;
    return t;
}
inline void startTiming() {
    msl_sync();
    timing_start() = wtime();
}
inline double splitTime(int) {
    msl_sync();
    double now = wtime(), d = now - timing_start();
    timing_start() = now;
    return d;
}
inline double stopTiming() {
    msl_sync();
    return wtime() - timing_start();
}
inline void printTimeToFile(const char *id, const char *file_name) {
    std::ofstream f(file_name, std::ios::app);
    f << id << ";" << stopTiming() << "\n";
}

}  // namespace msl
