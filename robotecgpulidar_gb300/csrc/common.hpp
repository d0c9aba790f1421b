// Host-side utilities of the C API layer: exception types mapped to rgl_status_t, field table,
// device buffers and a minimal logger.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <rgl/api/core.h>

namespace rgl {

// Exceptions and the status each maps to (reference src/api/apiCommon.hpp:55-106).
struct InvalidAPIArgument : std::invalid_argument
{
	using std::invalid_argument::invalid_argument; // RGL_INVALID_ARGUMENT
};
struct InvalidAPIObject : std::runtime_error
{
	using std::runtime_error::runtime_error; // RGL_INVALID_API_OBJECT
};
struct InvalidPipeline : std::runtime_error
{
	using std::runtime_error::runtime_error; // RGL_INVALID_PIPELINE
};
struct NotImplemented : std::runtime_error
{
	using std::runtime_error::runtime_error; // RGL_NOT_IMPLEMENTED
};

std::string format(const char* fmt, ...) __attribute__((format(printf, 1, 2)));

#define RGL_CHECK_CUDA(expr)                                                                                                   \
	do {                                                                                                                       \
		cudaError_t err_ = (expr);                                                                                             \
		if (err_ != cudaSuccess) {                                                                                             \
			throw std::runtime_error(::rgl::format("CUDA error: %s (%s) at %s:%d", cudaGetErrorString(err_), #expr, __FILE__, \
			                                       __LINE__));                                                                 \
		}                                                                                                                      \
	} while (0)

// ---- fields (reference src/RGLFields.hpp:108-201)
size_t fieldSize(rgl_field_t f);   // throws InvalidAPIArgument for unknown fields
bool isDummy(rgl_field_t f);       // paddings
const char* fieldName(rgl_field_t f);
size_t pointSize(const std::vector<rgl_field_t>& fields);

// ---- logging (reference src/Logger.cpp:17-59, reduced to level / file / stdout)
enum class LogLevel : int
{
	Trace = 0,
	Debug = 1,
	Info = 2,
	Warn = 3,
	Error = 4,
	Critical = 5,
	Off = 6
};
void logConfigure(int level, const char* filePath, bool useStdout);
void logMessage(LogLevel level, const std::string& msg);

// ---- device memory

// Incremented whenever any DeviceBuffer changes its device address; a captured CUDA graph of a run is
// replayed only while this value is unchanged.
uint64_t allocationEpoch();

// Grow-only device allocation owned by a node or scene.
class DeviceBuffer
{
public:
	DeviceBuffer() = default;
	// A buffer that kernels reach only through another device-resident pointer (scene data behind the
	// SceneView) does not invalidate captured runs when it moves.
	explicit DeviceBuffer(bool affectsCapturedRuns) : tracked_(affectsCapturedRuns) {}
	DeviceBuffer(const DeviceBuffer&) = delete;
	DeviceBuffer& operator=(const DeviceBuffer&) = delete;
	~DeviceBuffer();
	void* ensure(size_t bytes);
	void* get() const { return ptr_; }
	size_t capacity() const { return cap_; }
	void release();

	template<class T>
	T* as() const
	{
		return static_cast<T*>(ptr_);
	}

private:
	void* ptr_ = nullptr;
	size_t cap_ = 0;
	bool tracked_ = true;
};

// Error flag of a kernel (stack overflow, look-back timeout, ...). The flags of all nodes live in
// shared chunks of int32 slots in mapped pinned host memory: a kernel raises one with a plain store of
// 1 through the device address, and a completed run checks its flags by reading host memory, with no
// copy (result reads would otherwise pay one blocking device-to-host copy each).
class ErrorSlot
{
public:
	ErrorSlot() = default;
	ErrorSlot(const ErrorSlot&) = delete;
	ErrorSlot& operator=(const ErrorSlot&) = delete;
	~ErrorSlot();
	// Device address of the flag (zero when first handed out). Allocates: call outside stream capture.
	int32_t* device();
	// Value of the flag; valid once the work that may raise it has completed.
	bool raised() const;
	// Resets the flag (no work that may raise it may be running).
	void clear();

private:
	int chunk_ = -1;
	int index_ = -1;
};
// Orders the host's later reads of the flags after the completion it has just observed. Call after
// the work that may raise them has completed.
void refreshErrorSlots();

// Grow-only pinned host allocation.
class PinnedBuffer
{
public:
	PinnedBuffer() = default;
	PinnedBuffer(const PinnedBuffer&) = delete;
	PinnedBuffer& operator=(const PinnedBuffer&) = delete;
	~PinnedBuffer();
	void* ensure(size_t bytes);
	void* get() const { return ptr_; }

private:
	void* ptr_ = nullptr;
	size_t cap_ = 0;
};

// Library-wide CUDA state: device selected lazily on the first API call.
void ensureCudaInitialized();

// One parameter block's host-to-device copy, made by a gather kernel (kernels.hpp) instead of a
// copy node of its own.
struct ParamCopy
{
	const void* src; // pinned host memory
	void* dst;       // device memory
	uint32_t bytes;
	uint32_t pad;
};
// While non-null on this thread (during the capture of a batched frame), StagedParam::enqueue appends
// its copy here instead of issuing it; the capturing code then makes all of them in one kernel node
// placed before every other node of the graph.
extern thread_local std::vector<ParamCopy>* deferredParamCopies;

// A small parameter block (a transform, noise parameters) staged in pinned host memory before every
// run and copied to device memory by the run itself, so a captured run replayed later reads the
// current values. Call host() and device() in the prepare phase, enqueue() in the enqueue phase.
template<class T>
class StagedParam
{
public:
	T& host() { return *static_cast<T*>(h_.ensure(sizeof(T))); }
	const T* device() { return static_cast<const T*>(d_.ensure(sizeof(T))); }
	const T* enqueue(cudaStream_t s)
	{
		if (deferredParamCopies != nullptr) {
			deferredParamCopies->push_back(ParamCopy{h_.get(), d_.get(), (uint32_t) sizeof(T), 0});
		} else {
			RGL_CHECK_CUDA(cudaMemcpyAsync(d_.get(), h_.get(), sizeof(T), cudaMemcpyHostToDevice, s));
		}
		return d_.as<T>();
	}

private:
	PinnedBuffer h_;
	DeviceBuffer d_;
};

} // namespace rgl
