#include "common.hpp"

#include <atomic>
#include <cstring>
#include <iostream>

#include "kernels.hpp"

namespace rgl {

thread_local std::vector<ParamCopy>* deferredParamCopies = nullptr;

std::string format(const char* fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	char buf[1024];
	int n = vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	if (n < 0) {
		return {};
	}
	if ((size_t) n < sizeof(buf)) {
		return std::string(buf, n);
	}
	std::string out(n + 1, '\0');
	va_start(ap, fmt);
	vsnprintf(out.data(), out.size(), fmt, ap);
	va_end(ap);
	out.resize(n);
	return out;
}

size_t fieldSize(rgl_field_t f)
{
	switch (f) {
		case RGL_FIELD_XYZ_VEC3_F32: return 12;
		case RGL_FIELD_INTENSITY_F32: return 4;
		case RGL_FIELD_INTENSITY_U8: return 1;
		case RGL_FIELD_IS_HIT_I32: return 4;
		case RGL_FIELD_IS_GROUND_I32: return 4;
		case RGL_FIELD_RAY_IDX_U32: return 4;
		case RGL_FIELD_ENTITY_ID_I32: return 4;
		case RGL_FIELD_DISTANCE_F32: return 4;
		case RGL_FIELD_AZIMUTH_F32: return 4;
		case RGL_FIELD_ELEVATION_F32: return 4;
		case RGL_FIELD_RING_ID_U16: return 2;
		case RGL_FIELD_RETURN_TYPE_U8: return 1;
		case RGL_FIELD_TIME_STAMP_F64: return 8;
		case RGL_FIELD_TIME_STAMP_U32: return 4;
		case RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32: return 12;
		case RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32: return 12;
		case RGL_FIELD_RADIAL_SPEED_F32: return 4;
		case RGL_FIELD_POWER_F32: return 4;
		case RGL_FIELD_RCS_F32: return 4;
		case RGL_FIELD_NOISE_F32: return 4;
		case RGL_FIELD_SNR_F32: return 4;
		case RGL_FIELD_NORMAL_VEC3_F32: return 12;
		case RGL_FIELD_INCIDENT_ANGLE_F32: return 4;
		case RGL_FIELD_RAY_POSE_MAT3x4_F32: return 48;
		case RGL_FIELD_LASER_RETRO_F32: return 4;
		case RGL_FIELD_PADDING_8: return 1;
		case RGL_FIELD_PADDING_16: return 2;
		case RGL_FIELD_PADDING_32: return 4;
		default: break;
	}
	throw InvalidAPIArgument(format("getFieldSize: unknown RGL field %d", (int) f));
}

bool isDummy(rgl_field_t f) { return f == RGL_FIELD_PADDING_8 || f == RGL_FIELD_PADDING_16 || f == RGL_FIELD_PADDING_32; }

const char* fieldName(rgl_field_t f)
{
	switch (f) {
		case RGL_FIELD_XYZ_VEC3_F32: return "XYZ_VEC3_F32";
		case RGL_FIELD_INTENSITY_F32: return "INTENSITY_F32";
		case RGL_FIELD_INTENSITY_U8: return "INTENSITY_U8";
		case RGL_FIELD_IS_HIT_I32: return "IS_HIT_I32";
		case RGL_FIELD_IS_GROUND_I32: return "IS_GROUND_I32";
		case RGL_FIELD_RAY_IDX_U32: return "RAY_IDX_U32";
		case RGL_FIELD_ENTITY_ID_I32: return "ENTITY_ID_I32";
		case RGL_FIELD_DISTANCE_F32: return "DISTANCE_F32";
		case RGL_FIELD_AZIMUTH_F32: return "AZIMUTH_F32";
		case RGL_FIELD_ELEVATION_F32: return "ELEVATION_F32";
		case RGL_FIELD_RING_ID_U16: return "RING_ID_U16";
		case RGL_FIELD_RETURN_TYPE_U8: return "RETURN_TYPE_U8";
		case RGL_FIELD_TIME_STAMP_F64: return "TIME_STAMP_F64";
		case RGL_FIELD_TIME_STAMP_U32: return "TIME_STAMP_U32";
		case RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32: return "ABSOLUTE_VELOCITY_VEC3_F32";
		case RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32: return "RELATIVE_VELOCITY_VEC3_F32";
		case RGL_FIELD_RADIAL_SPEED_F32: return "RADIAL_SPEED_F32";
		case RGL_FIELD_POWER_F32: return "POWER_F32";
		case RGL_FIELD_RCS_F32: return "RCS_F32";
		case RGL_FIELD_NOISE_F32: return "NOISE_F32";
		case RGL_FIELD_SNR_F32: return "SNR_F32";
		case RGL_FIELD_NORMAL_VEC3_F32: return "NORMAL_VEC3_F32";
		case RGL_FIELD_INCIDENT_ANGLE_F32: return "INCIDENT_ANGLE_F32";
		case RGL_FIELD_RAY_POSE_MAT3x4_F32: return "RAY_POSE_MAT3x4_F32";
		case RGL_FIELD_LASER_RETRO_F32: return "LASER_RETRO_F32";
		case RGL_FIELD_PADDING_8: return "PADDING_8";
		case RGL_FIELD_PADDING_16: return "PADDING_16";
		case RGL_FIELD_PADDING_32: return "PADDING_32";
		case RGL_FIELD_DYNAMIC_FORMAT: return "DYNAMIC_FORMAT";
		default: return "UNKNOWN_FIELD";
	}
}

size_t pointSize(const std::vector<rgl_field_t>& fields)
{
	size_t s = 0;
	for (auto f : fields) {
		s += fieldSize(f);
	}
	return s;
}

// ---------------------------------------------------------------- logging

namespace {
std::mutex logMutex;
int logLevel = (int) LogLevel::Info;
bool logStdout = true;
FILE* logFile = nullptr;
const char* levelName(LogLevel l)
{
	static const char* names[] = {"trace", "debug", "info", "warning", "error", "critical", "off"};
	return names[(int) l];
}
} // namespace

void logConfigure(int level, const char* filePath, bool useStdout)
{
	std::lock_guard<std::mutex> g(logMutex);
	if (logFile) {
		fclose(logFile);
		logFile = nullptr;
	}
	logLevel = level;
	logStdout = useStdout;
	if (filePath != nullptr && filePath[0] != '\0') {
		logFile = fopen(filePath, "w");
		if (!logFile) {
			throw std::runtime_error(format("cannot open log file '%s'", filePath));
		}
	}
}

void logMessage(LogLevel level, const std::string& msg)
{
	std::lock_guard<std::mutex> g(logMutex);
	if ((int) level < logLevel || level == LogLevel::Off) {
		return;
	}
	if (logStdout) {
		fprintf(stdout, "[RGL] [%s] %s\n", levelName(level), msg.c_str());
		fflush(stdout);
	}
	if (logFile) {
		fprintf(logFile, "[%s] %s\n", levelName(level), msg.c_str());
		fflush(logFile);
	}
}

// ---------------------------------------------------------------- buffers

namespace {
std::atomic<uint64_t> allocEpoch{0};
}
uint64_t allocationEpoch() { return allocEpoch.load(std::memory_order_relaxed); }

DeviceBuffer::~DeviceBuffer() { release(); }

void DeviceBuffer::release()
{
	if (ptr_) {
		cudaFree(ptr_);
		if (tracked_) {
			allocEpoch.fetch_add(1, std::memory_order_relaxed);
		}
	}
	ptr_ = nullptr;
	cap_ = 0;
}

void* DeviceBuffer::ensure(size_t bytes)
{
	if (bytes <= cap_ && ptr_ != nullptr) {
		return ptr_;
	}
	size_t want = bytes < 256 ? 256 : bytes;
	void* p = nullptr;
	RGL_CHECK_CUDA(cudaMalloc(&p, want));
	if (ptr_) {
		cudaFree(ptr_);
	}
	ptr_ = p;
	cap_ = want;
	if (tracked_) {
		allocEpoch.fetch_add(1, std::memory_order_relaxed);
	}
	return ptr_;
}

PinnedBuffer::~PinnedBuffer()
{
	if (ptr_) {
		cudaFreeHost(ptr_);
	}
}

void* PinnedBuffer::ensure(size_t bytes)
{
	if (bytes <= cap_ && ptr_ != nullptr) {
		return ptr_;
	}
	size_t want = bytes < 256 ? 256 : bytes;
	void* p = nullptr;
	RGL_CHECK_CUDA(cudaMallocHost(&p, want));
	if (ptr_) {
		cudaFreeHost(ptr_);
	}
	ptr_ = p;
	cap_ = want;
	return ptr_;
}

// ---------------------------------------------------------------- error slots

namespace {
constexpr int kSlotsPerChunk = 4096;
struct SlotChunk
{
	int32_t* dev = nullptr;           // device address of `host` (mapped pinned memory)
	volatile int32_t* host = nullptr;
	int highWater = 0; // slots ever handed out
	std::vector<int> freeList;
};
std::mutex slotMutex;
// Never destroyed: slots owned by static objects (the default scene) are released during exit,
// possibly after function-local statics constructed later than them are gone.
std::vector<SlotChunk>& slotChunks()
{
	static auto* chunks = new std::vector<SlotChunk>();
	return *chunks;
}
} // namespace

ErrorSlot::~ErrorSlot()
{
	if (chunk_ < 0) {
		return;
	}
	std::lock_guard<std::mutex> g(slotMutex);
	slotChunks()[chunk_].freeList.push_back(index_); // zeroed again when handed out
}

int32_t* ErrorSlot::device()
{
	std::lock_guard<std::mutex> g(slotMutex);
	auto& chunks = slotChunks();
	if (chunk_ < 0) {
		int c = -1, i = -1;
		for (size_t k = 0; k < chunks.size() && c < 0; ++k) {
			if (!chunks[k].freeList.empty()) {
				c = (int) k;
				i = chunks[k].freeList.back();
				chunks[k].freeList.pop_back();
			} else if (chunks[k].highWater < kSlotsPerChunk) {
				c = (int) k;
				i = chunks[k].highWater++;
			}
		}
		if (c < 0) {
			SlotChunk n;
			void* h = nullptr;
			RGL_CHECK_CUDA(cudaHostAlloc(&h, sizeof(int32_t) * kSlotsPerChunk, cudaHostAllocMapped | cudaHostAllocPortable));
			std::memset(h, 0, sizeof(int32_t) * kSlotsPerChunk);
			void* d = nullptr;
			RGL_CHECK_CUDA(cudaHostGetDevicePointer(&d, h, 0));
			n.host = static_cast<volatile int32_t*>(h);
			n.dev = static_cast<int32_t*>(d);
			n.highWater = 1;
			chunks.push_back(std::move(n));
			c = (int) chunks.size() - 1;
			i = 0;
		}
		chunks[c].host[i] = 0;
		chunk_ = c;
		index_ = i;
	}
	return chunks[chunk_].dev + index_;
}

bool ErrorSlot::raised() const
{
	if (chunk_ < 0) {
		return false;
	}
	std::lock_guard<std::mutex> g(slotMutex);
	return slotChunks()[chunk_].host[index_] != 0;
}

void ErrorSlot::clear()
{
	if (chunk_ < 0) {
		return;
	}
	std::lock_guard<std::mutex> g(slotMutex);
	slotChunks()[chunk_].host[index_] = 0;
}

void refreshErrorSlots()
{
	// The kernels' stores to mapped memory are visible once their completion has been observed (an
	// event or stream synchronisation); the fence keeps the compiler and CPU from reading earlier.
	std::atomic_thread_fence(std::memory_order_acquire);
}

void ensureCudaInitialized()
{
	static bool done = false;
	if (done) {
		return;
	}
	int count = 0;
	cudaError_t e = cudaGetDeviceCount(&count);
	if (e != cudaSuccess || count == 0) {
		throw std::runtime_error(format("no CUDA device available (%s)", cudaGetErrorString(e)));
	}
	RGL_CHECK_CUDA(cudaSetDevice(0));
	RGL_CHECK_CUDA(cudaFree(nullptr));
	done = true;
}

// ---------------------------------------------------------------- launch counter

namespace {
std::atomic<uint64_t> launches{0};
}
void countLaunch(uint64_t n) { launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launchCount() { return launches.load(std::memory_order_relaxed); }

} // namespace rgl
