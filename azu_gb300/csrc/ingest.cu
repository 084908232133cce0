// Sensor-side frame ingest (host code): recordings written by libfreenect's
// fakenect-record (the reference's reader: tools/FakenectRecording.h:35-81),
// depth/RGB pairing with the rules of KinectSensor::onDepth / onRgb
// (src/sensor/KinectSensor.cpp:262-362: depth-led, nearest RGB within
// kMaxColorSkewMs = 17 ms of the 60 MHz device counter, else depth-only), and
// a ring of pinned host slots filled by a reader thread, each slot holding one
// frame's raw depth and RGB back to back so that a frame reaches the device in
// a single host-to-device copy (azu_pipeline_process_frame_packed).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "azu_internal.h"

namespace {

constexpr int kW = 640, kH = 480;
constexpr size_t kDepthBytes = size_t(kW) * kH * 2, kRgbBytes = size_t(kW) * kH * 3;
constexpr double kTicksPerMs = 60000.0, kMaxColorSkewMs = 17.0;

struct Entry {
    char type = 0;
    double host_s = 0.0;
    uint32_t ticks = 0;
    std::string file;
};

struct Frame {
    int depth = -1, rgb = -1;  // entry indices; rgb -1: depth-only
};

// Signed depth - rgb delta in ms, correct across a counter wrap.
double tick_delta_ms(uint32_t d, uint32_t r) { return static_cast<int32_t>(d - r) / kTicksPerMs; }

// The payload after the one-line PGM/PPM header.
bool read_payload(const std::string& path, size_t bytes, void* out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::string header;
    std::getline(f, header);
    f.read(static_cast<char*>(out), static_cast<std::streamsize>(bytes));
    return static_cast<size_t>(f.gcount()) == bytes;
}

}  // namespace

struct azu_recording {
    std::string dir;
    std::vector<Entry> entries;
    std::vector<Frame> frames;
};

struct azu_ingest {
    azu_recording* rec = nullptr;
    int slots = 0;
    uint8_t* ring = nullptr;        // pinned: slots x (depth | rgb)
    std::vector<int> frame_of;      // frame index held by each slot
    std::vector<int> rgb_valid;
    std::vector<int> ok;            // the payload was read completely
    int first = 0, end = 0;
    // head: next frame the reader fills; tail: next the consumer takes;
    // released: frames whose slots are free again
    int head = 0, tail = 0, released = 0;
    std::mutex m;
    std::condition_variable cv;
    bool stop = false;
    std::thread reader;
};

using namespace azu;

namespace {

// KinectSensor::onDepth / onRgb over the recording order (accelerometer
// samples do not take part in pairing). A depth frame still waiting for a
// nearer RGB sample when the recording ends is not published: the sensor fed
// the same samples parks it until a later sample arrives
// (src/sensor/KinectSensor.cpp:295-312), and none does.
void pair_entries(azu_recording* r) {
    int waiting = -1, held = -1;
    for (int i = 0; i < static_cast<int>(r->entries.size()); ++i) {
        const Entry& e = r->entries[i];
        if (e.type == 'd') {
            if (waiting >= 0) r->frames.push_back(Frame{waiting, -1});
            waiting = -1;
            if (held < 0) {
                waiting = i;
            } else {
                const double d = tick_delta_ms(e.ticks, r->entries[held].ticks);
                if (std::fabs(d) <= kMaxColorSkewMs) {
                    r->frames.push_back(Frame{i, held});
                    held = -1;
                } else if (d > 0.0) {
                    waiting = i;  // the newest RGB is too old; the next one is nearer
                } else {
                    r->frames.push_back(Frame{i, -1});
                }
            }
        } else if (e.type == 'r') {
            bool spent = false;
            if (waiting >= 0) {
                const double d = tick_delta_ms(r->entries[waiting].ticks, e.ticks);
                if (std::fabs(d) <= kMaxColorSkewMs) {
                    r->frames.push_back(Frame{waiting, i});
                    spent = true;
                } else {
                    r->frames.push_back(Frame{waiting, -1});
                }
                waiting = -1;
            }
            held = spent ? -1 : i;
        }
    }
}

bool read_frame(const azu_recording* r, int k, uint16_t* depth, uint8_t* rgb, int* rgb_valid) {
    const Frame& f = r->frames[k];
    if (!read_payload(r->dir + "/" + r->entries[f.depth].file, kDepthBytes, depth)) return false;
    const bool has_rgb = f.rgb >= 0;
    if (rgb) {
        if (has_rgb) {
            if (!read_payload(r->dir + "/" + r->entries[f.rgb].file, kRgbBytes, rgb)) return false;
        } else {
            std::memset(rgb, 0, kRgbBytes);
        }
    }
    if (rgb_valid) *rgb_valid = has_rgb ? 1 : 0;
    return true;
}

void reader_main(azu_ingest* g) {
    for (;;) {
        int k;
        {
            std::unique_lock<std::mutex> lk(g->m);
            g->cv.wait(lk, [g] { return g->stop || (g->head < g->end && g->head - g->released < g->slots); });
            if (g->stop || g->head >= g->end) return;
            k = g->head;
        }
        const int slot = (k - g->first) % g->slots;
        uint8_t* p = g->ring + static_cast<size_t>(slot) * (kDepthBytes + kRgbBytes);
        int rv = 0;
        const bool ok = read_frame(g->rec, k, reinterpret_cast<uint16_t*>(p), p + kDepthBytes, &rv);
        {
            std::lock_guard<std::mutex> lk(g->m);
            g->frame_of[slot] = k;
            g->rgb_valid[slot] = rv;
            g->ok[slot] = ok ? 1 : 0;
            g->head = k + 1;
        }
        g->cv.notify_all();
    }
}

}  // namespace

extern "C" int azu_recording_open(const char* dir, azu_recording** out) {
    AZU_CHECK_ARG(dir != nullptr && out != nullptr, "null argument");
    *out = nullptr;
    std::ifstream index(std::string(dir) + "/INDEX.txt");
    if (!index) {
        set_error("cannot open %s/INDEX.txt", dir);
        return AZU_E_INVALID;
    }
    azu_recording* r = new azu_recording();
    r->dir = dir;
    std::string line;
    while (std::getline(index, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        Entry e;
        unsigned int ticks = 0;
        if (line.size() < 3 || std::sscanf(line.c_str(), "%c-%lf-%u-", &e.type, &e.host_s, &ticks) != 3) continue;
        e.ticks = ticks;
        e.file = line;
        r->entries.push_back(std::move(e));
    }
    pair_entries(r);
    *out = r;
    return AZU_OK;
}

extern "C" void azu_recording_close(azu_recording* r) { delete r; }

extern "C" int azu_recording_frame_count(const azu_recording* r) {
    return r ? static_cast<int>(r->frames.size()) : 0;
}

extern "C" int azu_recording_frame_info(const azu_recording* r, int k, uint32_t* depth_ticks, uint32_t* rgb_ticks,
                                        int* rgb_valid) {
    AZU_CHECK_ARG(r != nullptr && k >= 0 && k < static_cast<int>(r->frames.size()), "frame index");
    const Frame& f = r->frames[k];
    if (depth_ticks) *depth_ticks = r->entries[f.depth].ticks;
    if (rgb_ticks) *rgb_ticks = f.rgb >= 0 ? r->entries[f.rgb].ticks : 0;
    if (rgb_valid) *rgb_valid = f.rgb >= 0 ? 1 : 0;
    return AZU_OK;
}

extern "C" int azu_recording_read(const azu_recording* r, int k, uint16_t* depth, uint8_t* rgb, int* rgb_valid) {
    AZU_CHECK_ARG(r != nullptr && depth != nullptr && k >= 0 && k < static_cast<int>(r->frames.size()),
                  "null argument / frame index");
    if (!read_frame(r, k, depth, rgb, rgb_valid)) {
        set_error("short or missing payload for frame %d", k);
        return AZU_E_INVALID;
    }
    return AZU_OK;
}

extern "C" int azu_ingest_create(azu_recording* rec, int slots, int first, int count, azu_ingest** out) {
    AZU_CHECK_ARG(rec != nullptr && out != nullptr && slots >= 1 && slots <= 256, "null argument / slots");
    const int n = static_cast<int>(rec->frames.size());
    AZU_CHECK_ARG(first >= 0 && first <= n && count >= 0, "frame range");
    *out = nullptr;
    azu_ingest* g = new azu_ingest();
    g->rec = rec;
    g->slots = slots;
    g->first = g->head = g->tail = g->released = first;
    g->end = std::min(n, first + count);
    g->frame_of.assign(slots, -1);
    g->rgb_valid.assign(slots, 0);
    g->ok.assign(slots, 0);
    const cudaError_t e = cudaHostAlloc(&g->ring, static_cast<size_t>(slots) * (kDepthBytes + kRgbBytes),
                                        cudaHostAllocDefault);
    if (e != cudaSuccess) {
        set_error("pinned ring: %s", cudaGetErrorString(e));
        delete g;
        return AZU_E_NOMEM;
    }
    g->reader = std::thread(reader_main, g);
    *out = g;
    return AZU_OK;
}

extern "C" int azu_ingest_destroy(azu_ingest* g) {
    if (!g) return AZU_OK;
    {
        std::lock_guard<std::mutex> lk(g->m);
        g->stop = true;
    }
    g->cv.notify_all();
    if (g->reader.joinable()) g->reader.join();
    if (g->ring) cudaFreeHost(g->ring);
    delete g;
    return AZU_OK;
}

// The next frame in order: a pinned slot holding depth (640x480 uint16) then
// RGB (640x480x3). Blocks until the reader has it. Returns 1 (and no slot) at
// the end of the range.
extern "C" int azu_ingest_next(azu_ingest* g, const void** slot, int* frame_index, int* rgb_valid) {
    AZU_CHECK_ARG(g != nullptr && slot != nullptr, "null argument");
    std::unique_lock<std::mutex> lk(g->m);
    if (g->tail >= g->end) return 1;
    AZU_CHECK_ARG(g->tail - g->released < g->slots, "release consumed slots before taking more than the ring holds");
    g->cv.wait(lk, [g] { return g->head > g->tail; });
    const int s = (g->tail - g->first) % g->slots;
    if (!g->ok[s]) {
        set_error("short or missing payload for frame %d", g->tail);
        return AZU_E_INVALID;
    }
    *slot = g->ring + static_cast<size_t>(s) * (kDepthBytes + kRgbBytes);
    if (frame_index) *frame_index = g->frame_of[s];
    if (rgb_valid) *rgb_valid = g->rgb_valid[s];
    g->tail++;
    return AZU_OK;
}

// Returns the oldest consumed slot to the reader.
extern "C" int azu_ingest_release(azu_ingest* g) {
    AZU_CHECK_ARG(g != nullptr, "null argument");
    {
        std::lock_guard<std::mutex> lk(g->m);
        AZU_CHECK_ARG(g->released < g->tail, "nothing to release");
        g->released++;
    }
    g->cv.notify_all();
    return AZU_OK;
}
