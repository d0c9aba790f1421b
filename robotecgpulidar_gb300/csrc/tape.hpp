// Tape: recording of API calls to a YAML + binary file pair and their playback (reference
// src/tape/TapeRecorder.hpp:28-151, TapePlayer.cpp:27-150, PlaybackState.cpp:28-86, API
// include/rgl/api/extensions/tape.h:26-45).
//
// Format (kept identical to the reference's so tapes move between the two libraries):
//  * <path>.yaml is a block sequence with one item per call, `- <function>: {t: <ns since the
//    recording began>, a: [<args>]}`; the first item is rgl_get_version_info with the library version;
//  * handles (meshes, entities, nodes, textures, scenes) are recorded as integers (their address at
//    recording time) and mapped to the handles the playback creates;
//  * arrays, and single vec3 / mat3x4 arguments passed by pointer, go to <path>.bin, each starting at
//    a 16-byte boundary (zero padding); the YAML holds their byte offset;
//  * enums, integers, floats and booleans are written as scalars; out-parameters (counts, priorities,
//    version numbers) as the value they received.
#pragma once

#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>

#include <rgl/api/core.h>

namespace rgl {
namespace tape {

// Failures of recording or playback: reported as RGL_TAPE_ERROR.
struct RecordError : std::runtime_error
{
	using std::runtime_error::runtime_error;
};
// A tape file that cannot be opened: RGL_INVALID_FILE_PATH.
struct InvalidFilePath : std::runtime_error
{
	using std::runtime_error::runtime_error;
};

bool recording();
void beginRecording(const char* path);
void endRecording();
// Appends one call; `args` are the YAML scalars of its arguments.
void record(const char* fn, std::initializer_list<std::string> args);

// Argument encoders (valid only while recording: bin() appends to the binary file).
std::string handle(const void* h);
std::string num(int64_t v);
std::string unum(uint64_t v);
std::string real(float v);
std::string real(double v);
std::string real(double v, int significantDigits);
float parseFloat(const std::string& s);
std::string flag(bool v);
std::string text(const char* s);
std::string bin(const void* data, size_t bytes);
template<class T>
std::string arr(const T* data, int64_t count)
{
	return bin(data, data != nullptr && count > 0 ? sizeof(T) * (size_t) count : 0);
}

// Plays a tape, pacing the calls by their recorded timestamps (reference playApproximatelyRealtime).
void play(const char* path);

// Logs a failed recording of `fn` (the API call itself has completed).
void recordFailed(const char* fn, const char* why);

} // namespace tape
} // namespace rgl

// Records the calling API function with the given argument encodings when a recording is active.
#define RGL_TAPE_RECORD(...)                                                                                                   \
	do {                                                                                                                       \
		if (::rgl::tape::recording()) {                                                                                        \
			try {                                                                                                              \
				::rgl::tape::record(__func__, {__VA_ARGS__});                                                                  \
			}                                                                                                                  \
			catch (std::exception & e) {                                                                                       \
				::rgl::tape::recordFailed(__func__, e.what());                                                                 \
			}                                                                                                                  \
		}                                                                                                                      \
	} while (0)
