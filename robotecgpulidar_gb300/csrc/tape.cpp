#include "tape.hpp"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cctype>
#include <cerrno>
#include <cmath>
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <functional>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <rgl/api/extensions/tape.h>

#include "common.hpp"

namespace rgl {
namespace tape {

namespace {

// Oldest tape format this player reads (reference src/tape/tapeDefinitions.hpp:19-21).
constexpr int kFormatMajor = 0, kFormatMinor = 16, kFormatPatch = 3;

struct Recorder
{
	FILE* yaml = nullptr;
	FILE* binFile = nullptr;
	size_t binOffset = 0;
	std::chrono::steady_clock::time_point t0;
};

std::unique_ptr<Recorder>& active()
{
	static std::unique_ptr<Recorder> r;
	return r;
}

// True while play() runs: calls made by the playback are not recorded again.
bool& playing()
{
	static bool p = false;
	return p;
}

} // namespace

bool recording() { return active() != nullptr && !playing(); }

void beginRecording(const char* path)
{
	if (active()) {
		throw RecordError("rgl_tape_record_begin: recording already active");
	}
	auto r = std::make_unique<Recorder>();
	const std::string binPath = std::string(path) + ".bin", yamlPath = std::string(path) + ".yaml";
	r->binFile = std::fopen(binPath.c_str(), "wb");
	if (r->binFile == nullptr) {
		throw InvalidFilePath(format("rgl_tape_record_begin: could not open binary file '%s' due to the error: %s", binPath.c_str(),
		                             std::strerror(errno)));
	}
	r->yaml = std::fopen(yamlPath.c_str(), "w");
	if (r->yaml == nullptr) {
		std::fclose(r->binFile);
		throw InvalidFilePath(format("rgl_tape_record_begin: could not open yaml file '%s' due to the error: %s", yamlPath.c_str(),
		                             std::strerror(errno)));
	}
	r->t0 = std::chrono::steady_clock::now();
	active() = std::move(r);
	int32_t major = 0, minor = 0, patch = 0;
	rgl_get_version_info(&major, &minor, &patch); // records itself: the tape's first item
}

void endRecording()
{
	if (!active()) {
		throw RecordError("rgl_tape_record_end: no recording active");
	}
	std::unique_ptr<Recorder> r = std::move(active());
	const bool ok = std::fflush(r->yaml) == 0 && std::fflush(r->binFile) == 0;
	std::fclose(r->yaml);
	std::fclose(r->binFile);
	if (!ok) {
		throw RecordError("rgl_tape_record_end: failed to flush the tape files");
	}
}

void record(const char* fn, std::initializer_list<std::string> args)
{
	Recorder& r = *active();
	const long long ns =
	    (long long) std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - r.t0).count();
	std::string line = "- ";
	line += fn;
	line += ": {t: " + std::to_string(ns) + ", a: [";
	bool first = true;
	for (const auto& a : args) {
		if (!first) {
			line += ", ";
		}
		line += a;
		first = false;
	}
	line += "]}\n";
	if (std::fputs(line.c_str(), r.yaml) < 0) {
		throw RecordError("failed to write the tape's yaml file");
	}
}

void recordFailed(const char* fn, const char* why)
{
	logMessage(LogLevel::Error, format("tape: failed to record %s: %s", fn, why));
}

std::string handle(const void* h) { return std::to_string((uint64_t) (uintptr_t) h); }
std::string num(int64_t v) { return std::to_string(v); }
std::string unum(uint64_t v) { return std::to_string(v); }
// Floats as yaml-cpp's emitter writes them (the reference recorder's): shortest-round-trip digits
// (9 significant for float, 17 for double) in %g form, and the YAML spellings .inf, -.inf, .nan.
std::string real(float v) { return real((double) v, 9); }
std::string real(double v) { return real(v, 17); }
std::string real(double v, int digits)
{
	if (std::isnan(v)) {
		return ".nan";
	}
	if (std::isinf(v)) {
		return v > 0 ? ".inf" : "-.inf";
	}
	char b[40];
	std::snprintf(b, sizeof(b), "%.*g", digits, v);
	return b;
}

// A float argument: plain decimal, or a YAML special (.inf, -.inf, +.inf, .nan in any of the YAML
// core schema's capitalisations), as a tape from either recorder holds it.
float parseFloat(const std::string& s)
{
	std::string t = s;
	for (auto& ch : t) {
		ch = (char) std::tolower((unsigned char) ch);
	}
	if (t == ".inf" || t == "+.inf") {
		return INFINITY;
	}
	if (t == "-.inf") {
		return -INFINITY;
	}
	if (t == ".nan") {
		return NAN;
	}
	return std::strtof(s.c_str(), nullptr);
}
std::string flag(bool v) { return v ? "true" : "false"; }
std::string text(const char* s)
{
	if (s == nullptr) {
		return "~";
	}
	std::string out = "\"";
	for (const char* p = s; *p; ++p) {
		if (*p == '"' || *p == '\\') {
			out += '\\';
		}
		out += *p;
	}
	return out + "\"";
}

std::string bin(const void* data, size_t bytes)
{
	Recorder& r = *active();
	const size_t at = r.binOffset;
	if (bytes > 0 && std::fwrite(data, 1, bytes, r.binFile) != bytes) {
		throw RecordError("Failed to write data to binary file");
	}
	const size_t pad = (16 - bytes % 16) % 16;
	static const uint8_t zeros[16] = {};
	if (pad > 0 && std::fwrite(zeros, 1, pad, r.binFile) != pad) {
		throw RecordError("Failed to write data to binary file");
	}
	r.binOffset += bytes + pad;
	return std::to_string(at);
}

// ---------------------------------------------------------------- playback

namespace {

// One recorded call: function name, timestamp and argument scalars (quotes removed from strings,
// `~` / `null` kept as written).
struct Call
{
	std::string fn;
	long long ns = 0;
	std::vector<std::string> args;
	std::vector<bool> quoted;
};

std::string trim(const std::string& s)
{
	size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
	return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// Splits a flow sequence body at top-level commas, honouring quotes.
void splitArgs(const std::string& body, Call& c)
{
	std::string cur;
	bool inQuote = false, wasQuoted = false;
	char q = 0;
	int depth = 0;
	auto flush = [&]() {
		std::string t = wasQuoted ? cur : trim(cur);
		if (!t.empty() || wasQuoted) {
			c.args.push_back(t);
			c.quoted.push_back(wasQuoted);
		}
		cur.clear();
		wasQuoted = false;
	};
	for (size_t i = 0; i < body.size(); ++i) {
		const char ch = body[i];
		if (inQuote) {
			if (q == '"' && ch == '\\' && i + 1 < body.size()) {
				cur += body[++i];
			} else if (ch == q) {
				if (q == '\'' && i + 1 < body.size() && body[i + 1] == '\'') {
					cur += '\'';
					++i;
				} else {
					inQuote = false;
				}
			} else {
				cur += ch;
			}
			continue;
		}
		if ((ch == '"' || ch == '\'') && trim(cur).empty()) {
			inQuote = true;
			wasQuoted = true;
			q = ch;
			cur.clear();
		} else if (ch == '[' || ch == '{') {
			++depth;
			cur += ch;
		} else if (ch == ']' || ch == '}') {
			--depth;
			cur += ch;
		} else if (ch == ',' && depth == 0) {
			flush();
		} else {
			cur += ch;
		}
	}
	flush();
}

// Parses `- fn: {t: N, a: [...]}` items; an item may continue over several lines.
std::vector<Call> parseYaml(const std::string& path)
{
	std::ifstream in(path);
	if (!in) {
		throw InvalidFilePath(format("TAPE: could not open yaml file: '%s'", path.c_str()));
	}
	std::vector<std::string> items;
	std::string line;
	while (std::getline(in, line)) {
		if (line.rfind("- ", 0) == 0) {
			items.push_back(line.substr(2));
		} else if (!trim(line).empty() && !items.empty()) {
			items.back() += " " + trim(line);
		} else if (!trim(line).empty() && trim(line) != "---") {
			throw RecordError("Unsupported Tape format: Detected outdated format");
		}
	}
	if (items.empty()) {
		throw RecordError("Invalid Tape: Empty YAML file detected");
	}
	std::vector<Call> calls;
	for (const auto& it : items) {
		Call c;
		const size_t colon = it.find(':');
		const size_t open = it.find('{', colon);
		const size_t close = it.rfind('}');
		if (colon == std::string::npos || open == std::string::npos || close == std::string::npos || close < open) {
			throw RecordError(format("TAPE: malformed call '%s'", it.c_str()));
		}
		c.fn = trim(it.substr(0, colon));
		const std::string inner = it.substr(open + 1, close - open - 1);
		const size_t tk = inner.find("t:");
		const size_t ak = inner.find("a:");
		if (tk == std::string::npos || ak == std::string::npos) {
			throw RecordError(format("TAPE: malformed call '%s'", it.c_str()));
		}
		c.ns = std::strtoll(inner.c_str() + tk + 2, nullptr, 10);
		const size_t lb = inner.find('[', ak), rb = inner.rfind(']');
		if (lb == std::string::npos || rb == std::string::npos || rb < lb) {
			throw RecordError(format("TAPE: malformed arguments of '%s'", c.fn.c_str()));
		}
		splitArgs(inner.substr(lb + 1, rb - lb - 1), c);
		calls.push_back(std::move(c));
	}
	return calls;
}

struct BinMap
{
	uint8_t* data = nullptr;
	size_t size = 0;
	explicit BinMap(const std::string& path)
	{
		const int fd = open(path.c_str(), O_RDONLY);
		if (fd < 0) {
			throw InvalidFilePath(
			    format("TAPE: could not open binary file: '%s'  due to the error: %s", path.c_str(), std::strerror(errno)));
		}
		struct stat sb
		{};
		if (fstat(fd, &sb) < 0) {
			close(fd);
			throw InvalidFilePath("TAPE: couldn't read binary file length");
		}
		size = (size_t) sb.st_size;
		if (size > 0) {
			void* p = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
			if (p == MAP_FAILED) {
				close(fd);
				throw InvalidFilePath(format("TAPE: could not mmap binary file: %s", path.c_str()));
			}
			data = static_cast<uint8_t*>(p);
		}
		close(fd);
	}
	~BinMap()
	{
		if (data) {
			munmap(data, size);
		}
	}
};

struct Playback
{
	const BinMap& bin;
	std::unordered_map<uint64_t, rgl_mesh_t> meshes;
	std::unordered_map<uint64_t, rgl_entity_t> entities;
	std::unordered_map<uint64_t, rgl_node_t> nodes;
	std::unordered_map<uint64_t, rgl_texture_t> textures;

	const Call* c = nullptr;
	const std::string& a(size_t i) const
	{
		if (i >= c->args.size()) {
			throw RecordError(format("TAPE: call %s has too few arguments", c->fn.c_str()));
		}
		return c->args[i];
	}
	uint64_t id(size_t i) const { return std::strtoull(a(i).c_str(), nullptr, 10); }
	int64_t i64(size_t i) const { return std::strtoll(a(i).c_str(), nullptr, 10); }
	int32_t i32(size_t i) const { return (int32_t) i64(i); }
	float f32(size_t i) const { return parseFloat(a(i)); }
	bool b(size_t i) const { return a(i) == "true" || a(i) == "True" || a(i) == "1"; }
	template<class T>
	const T* ptr(size_t i) const
	{
		const uint64_t off = id(i);
		if (off > bin.size) {
			throw RecordError(format("TAPE: binary offset %" PRIu64 " of %s is outside the file", off, c->fn.c_str()));
		}
		return reinterpret_cast<const T*>(bin.data + off);
	}
	// A handle argument: 0 is NULL; unknown ids are the recording's handles of objects this playback
	// never created (calls that failed while recording).
	template<class H>
	static H look(const std::unordered_map<uint64_t, H>& m, uint64_t key)
	{
		auto it = m.find(key);
		return it == m.end() ? nullptr : it->second;
	}
	rgl_node_t node(size_t i) const { return look(nodes, id(i)); }
	rgl_entity_t entity(size_t i) const { return look(entities, id(i)); }
	rgl_mesh_t mesh(size_t i) const { return look(meshes, id(i)); }
	rgl_texture_t texture(size_t i) const { return look(textures, id(i)); }
	// Create-or-modify node calls: the node recorded under the id, created at its first call.
	template<class Fn>
	void nodeCall(Fn&& fn)
	{
		const uint64_t key = id(0);
		rgl_node_t n = look(nodes, key);
		fn(&n);
		if (n != nullptr && key != 0) {
			nodes[key] = n;
		}
	}
};

using Player = std::function<void(Playback&)>;

const std::map<std::string, Player>& players()
{
	static const std::map<std::string, Player> m = {
	    {"rgl_get_version_info", [](Playback&) {}},
	    {"rgl_get_extension_info", [](Playback& p) { int32_t v = 0; rgl_get_extension_info((rgl_extension_t) p.i32(0), &v); }},
	    {"rgl_configure_logging",
	     [](Playback& p) {
		     const bool nullPath = !p.c->quoted[1] && (p.a(1) == "~" || p.a(1) == "null" || p.a(1).empty());
		     rgl_configure_logging((rgl_log_level_t) p.i32(0), nullPath ? nullptr : p.a(1).c_str(), p.b(2));
	     }},
	    {"rgl_cleanup",
	     [](Playback& p) {
		     rgl_cleanup();
		     p.meshes.clear();
		     p.entities.clear();
		     p.nodes.clear();
		     p.textures.clear();
	     }},
	    {"rgl_mesh_create",
	     [](Playback& p) {
		     rgl_mesh_t m = nullptr;
		     rgl_mesh_create(&m, p.ptr<rgl_vec3f>(1), p.i32(2), p.ptr<rgl_vec3i>(3), p.i32(4));
		     p.meshes[p.id(0)] = m;
	     }},
	    {"rgl_mesh_set_texture_coords", [](Playback& p) { rgl_mesh_set_texture_coords(p.mesh(0), p.ptr<rgl_vec2f>(1), p.i32(2)); }},
	    {"rgl_mesh_set_bone_weights",
	     [](Playback& p) { rgl_mesh_set_bone_weights(p.mesh(0), p.ptr<rgl_bone_weights_t>(1), p.i32(2)); }},
	    {"rgl_mesh_set_restposes", [](Playback& p) { rgl_mesh_set_restposes(p.mesh(0), p.ptr<rgl_mat3x4f>(1), p.i32(2)); }},
	    {"rgl_entity_set_pose_world", [](Playback& p) { rgl_entity_set_pose_world(p.entity(0), p.ptr<rgl_mat3x4f>(1), p.i32(2)); }},
	    {"rgl_entity_apply_external_animation",
	     [](Playback& p) { rgl_entity_apply_external_animation(p.entity(0), p.ptr<rgl_vec3f>(1), p.i32(2)); }},
	    {"rgl_texture_create",
	     [](Playback& p) {
		     rgl_texture_t t = nullptr;
		     rgl_texture_create(&t, p.ptr<void>(1), p.i32(2), p.i32(3));
		     p.textures[p.id(0)] = t;
	     }},
	    {"rgl_texture_destroy",
	     [](Playback& p) {
		     rgl_texture_destroy(p.texture(0));
		     p.textures.erase(p.id(0));
	     }},
	    {"rgl_texture_is_alive", [](Playback& p) { bool v = false; rgl_texture_is_alive(p.texture(0), &v); }},
	    {"rgl_entity_set_intensity_texture", [](Playback& p) { rgl_entity_set_intensity_texture(p.entity(0), p.texture(1)); }},
	    {"rgl_mesh_destroy",
	     [](Playback& p) {
		     rgl_mesh_destroy(p.mesh(0));
		     p.meshes.erase(p.id(0));
	     }},
	    {"rgl_mesh_is_alive", [](Playback& p) { bool v = false; rgl_mesh_is_alive(p.mesh(0), &v); }},
	    {"rgl_entity_create",
	     [](Playback& p) {
		     rgl_entity_t e = nullptr;
		     rgl_entity_create(&e, nullptr, p.mesh(2)); // tapes hold the default scene only
		     p.entities[p.id(0)] = e;
	     }},
	    {"rgl_entity_destroy",
	     [](Playback& p) {
		     rgl_entity_destroy(p.entity(0));
		     p.entities.erase(p.id(0));
	     }},
	    {"rgl_entity_set_transform", [](Playback& p) { rgl_entity_set_transform(p.entity(0), p.ptr<rgl_mat3x4f>(1)); }},
	    {"rgl_entity_set_id", [](Playback& p) { rgl_entity_set_id(p.entity(0), p.i32(1)); }},
	    {"rgl_entity_set_laser_retro", [](Playback& p) { rgl_entity_set_laser_retro(p.entity(0), p.f32(1)); }},
	    {"rgl_entity_is_alive", [](Playback& p) { bool v = false; rgl_entity_is_alive(p.entity(0), &v); }},
	    {"rgl_scene_set_time", [](Playback& p) { rgl_scene_set_time(nullptr, (uint64_t) p.id(1)); }},
	    {"rgl_graph_run", [](Playback& p) { rgl_graph_run(p.node(0)); }},
	    {"rgl_graph_destroy",
	     [](Playback& p) {
		     rgl_graph_destroy(p.node(0));
		     p.nodes.erase(p.id(0));
	     }},
	    {"rgl_graph_get_result_size",
	     [](Playback& p) {
		     int32_t n = 0, s = 0;
		     rgl_graph_get_result_size(p.node(0), (rgl_field_t) p.i32(1), &n, &s);
		     if (n != p.i32(2) || s != p.i32(3)) {
			     logMessage(LogLevel::Warn, format("tape_graph_get_result_size: actual (count %d, size %d) differs from tape (%d, %d)", n, s,
			                                       p.i32(2), p.i32(3)));
		     }
	     }},
	    {"rgl_graph_get_result_data",
	     [](Playback& p) {
		     rgl_node_t n = p.node(0);
		     const auto f = (rgl_field_t) p.i32(1);
		     int32_t count = 0, size = 0;
		     if (rgl_graph_get_result_size(n, f, &count, &size) == RGL_SUCCESS && count > 0) {
			     std::vector<char> tmp((size_t) count * (size_t) size);
			     rgl_graph_get_result_data(n, f, tmp.data());
		     }
	     }},
	    {"rgl_graph_node_add_child", [](Playback& p) { rgl_graph_node_add_child(p.node(0), p.node(1)); }},
	    {"rgl_graph_node_remove_child", [](Playback& p) { rgl_graph_node_remove_child(p.node(0), p.node(1)); }},
	    {"rgl_graph_node_set_priority", [](Playback& p) { rgl_graph_node_set_priority(p.node(0), p.i32(1)); }},
	    {"rgl_graph_node_get_priority", [](Playback& p) { int32_t v = 0; rgl_graph_node_get_priority(p.node(0), &v); }},
	    {"rgl_node_rays_from_mat3x4f",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_rays_from_mat3x4f(n, p.ptr<rgl_mat3x4f>(1), p.i32(2)); }); }},
	    {"rgl_node_rays_set_ring_ids",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_rays_set_ring_ids(n, p.ptr<int32_t>(1), p.i32(2)); }); }},
	    {"rgl_node_rays_set_range",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_rays_set_range(n, p.ptr<rgl_vec2f>(1), p.i32(2)); }); }},
	    {"rgl_node_rays_set_time_offsets",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_rays_set_time_offsets(n, p.ptr<float>(1), p.i32(2)); }); }},
	    {"rgl_node_rays_transform",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_rays_transform(n, p.ptr<rgl_mat3x4f>(1)); }); }},
	    {"rgl_node_points_transform",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_transform(n, p.ptr<rgl_mat3x4f>(1)); }); }},
	    {"rgl_node_raytrace", [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_raytrace(n, nullptr); }); }},
	    {"rgl_node_raytrace_configure_velocity",
	     [](Playback& p) { rgl_node_raytrace_configure_velocity(p.node(0), p.ptr<rgl_vec3f>(1), p.ptr<rgl_vec3f>(2)); }},
	    {"rgl_node_raytrace_configure_distortion", [](Playback& p) { rgl_node_raytrace_configure_distortion(p.node(0), p.b(1)); }},
	    {"rgl_node_raytrace_configure_non_hits",
	     [](Playback& p) { rgl_node_raytrace_configure_non_hits(p.node(0), p.f32(1), p.f32(2)); }},
	    {"rgl_node_raytrace_configure_mask",
	     [](Playback& p) { rgl_node_raytrace_configure_mask(p.node(0), p.ptr<int8_t>(1), p.i32(2)); }},
	    {"rgl_node_raytrace_configure_beam_divergence",
	     [](Playback& p) { rgl_node_raytrace_configure_beam_divergence(p.node(0), p.f32(1), p.f32(2)); }},
	    {"rgl_node_raytrace_configure_default_intensity",
	     [](Playback& p) { rgl_node_raytrace_configure_default_intensity(p.node(0), p.f32(1)); }},
	    {"rgl_node_raytrace_configure_return_mode",
	     [](Playback& p) { rgl_node_raytrace_configure_return_mode(p.node(0), (rgl_return_mode_t) p.i32(1)); }},
	    {"rgl_node_points_format",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_format(n, p.ptr<rgl_field_t>(1), p.i32(2)); }); }},
	    {"rgl_node_points_yield",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_yield(n, p.ptr<rgl_field_t>(1), p.i32(2)); }); }},
	    {"rgl_node_points_compact_by_field",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_compact_by_field(n, (rgl_field_t) p.i32(1)); }); }},
	    {"rgl_node_points_spatial_merge",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_spatial_merge(n, p.ptr<rgl_field_t>(1), p.i32(2)); }); }},
	    {"rgl_node_points_temporal_merge",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_temporal_merge(n, p.ptr<rgl_field_t>(1), p.i32(2)); }); }},
	    {"rgl_node_points_from_array",
	     [](Playback& p) {
		     p.nodeCall([&](rgl_node_t* n) { rgl_node_points_from_array(n, p.ptr<void>(1), p.i32(2), p.ptr<rgl_field_t>(3), p.i32(4)); });
	     }},
	    {"rgl_node_points_filter_ground",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_points_filter_ground(n, p.ptr<rgl_vec3f>(1), p.f32(2)); }); }},
	    {"rgl_node_gaussian_noise_angular_ray",
	     [](Playback& p) {
		     p.nodeCall([&](rgl_node_t* n) { rgl_node_gaussian_noise_angular_ray(n, p.f32(1), p.f32(2), (rgl_axis_t) p.i32(3)); });
	     }},
	    {"rgl_node_gaussian_noise_angular_hitpoint",
	     [](Playback& p) {
		     p.nodeCall([&](rgl_node_t* n) { rgl_node_gaussian_noise_angular_hitpoint(n, p.f32(1), p.f32(2), (rgl_axis_t) p.i32(3)); });
	     }},
	    {"rgl_node_gaussian_noise_distance",
	     [](Playback& p) { p.nodeCall([&](rgl_node_t* n) { rgl_node_gaussian_noise_distance(n, p.f32(1), p.f32(2), p.f32(3)); }); }},
	    {"rgl_node_is_alive", [](Playback& p) { bool v = false; rgl_node_is_alive(p.node(0), &v); }},
	};
	return m;
}

} // namespace

void play(const char* path)
{
	if (active()) {
		throw RecordError("rgl_tape_play: recording active");
	}
	const std::vector<Call> calls = parseYaml(std::string(path) + ".yaml");
	BinMap bin(std::string(path) + ".bin");
	// Reference src/tape/TapePlayer.cpp:48-63: the tape must carry a version record not older than
	// the format this player reads.
	const Call* version = nullptr;
	for (const auto& c : calls) {
		if (c.fn == "rgl_get_version_info") {
			version = &c;
			break;
		}
	}
	if (version == nullptr || version->args.size() < 3) {
		throw RecordError("Unsupported Tape format: Missing version record in the Tape");
	}
	const long long linear = 1000000ll * std::atoll(version->args[0].c_str()) + 1000ll * std::atoll(version->args[1].c_str()) +
	                         std::atoll(version->args[2].c_str());
	if (linear < 1000000ll * kFormatMajor + 1000ll * kFormatMinor + kFormatPatch) {
		throw RecordError(format("Unsupported Tape Format: Tape version is too old. Required version: %d.%d.%d.", kFormatMajor,
		                         kFormatMinor, kFormatPatch));
	}
	for (const auto& c : calls) {
		if (!players().count(c.fn)) {
			throw RecordError(format("unknown function to play: %s", c.fn.c_str()));
		}
	}
	Playback pb{bin};
	struct Guard
	{
		Guard() { playing() = true; }
		~Guard() { playing() = false; }
	} guard;
	const auto t0 = std::chrono::steady_clock::now();
	for (const auto& c : calls) {
		const auto due = t0 + std::chrono::nanoseconds(c.ns);
		std::this_thread::sleep_until(due);
		pb.c = &c;
		players().at(c.fn)(pb);
	}
}

} // namespace tape
} // namespace rgl
