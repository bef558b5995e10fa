// xtg_npy.cpp — xt::load_npy / xt::dump_npy between .npy files (or host
// buffers) and device memory (include/xtensor/io/xnpy.hpp:237-450, 674-800).
//
// Format (NumPy's .npy, as the reference reads and writes it):
//   "\x93NUMPY", major, minor, header length (2 bytes LE in 1.0, 4 in 2.0),
//   a Python-dict header "{'descr': '<f8', 'fortran_order': False,
//   'shape': (3, 3, 3), }" padded with spaces and ended by '\n' so that the
//   data starts on a 64-byte boundary, then the raw elements.
//
// Data path: the header is parsed on the calling thread; the data moves in
// 4 MiB chunks through pinned staging buffers.  Each of W host threads (up to
// 16) owns a CUDA
// stream and two buffers: it reads chunk k (pread from the file, or memcpy
// from a pageable host buffer) into one buffer while the copy of chunk k-1
// from the other is in flight, so the file read, the staging copy and the
// link transfer overlap across threads.  Saving runs the same ring backwards
// (device -> buffer -> file).  Buffered writes to one file serialise on the
// file's lock, so the write side depends on the file system: on tmpfs the
// file is sized, mapped, and every thread copies its chunks into the mapping
// (the page faults run in parallel); elsewhere one thread writes the chunks
// in order into a preallocated file while the next chunk's copy is in flight.  A destination with other strides than
// the file's order receives the bytes in a temporary first and is assigned
// from it (the device assign kernels do the reordering).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/vfs.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "xtg_plan.h"

namespace xtgh {

namespace {

const char kMagic[] = "\x93NUMPY";
constexpr size_t kMagicLen = 6;

bool host_little_endian() {
    const uint16_t one = 1;
    unsigned char c;
    memcpy(&c, &one, 1);
    return c == 1;
}

// The typestring the reference's build_typestring<T>() gives for each dtype
// (xnpy.hpp:77-188): endianness char ('|' for one-byte types), kind, size.
std::string typestring(int dtype) {
    char kind;
    switch (dtype) {
        case XTG_BOOL: kind = 'b'; break;
        case XTG_INT8: case XTG_INT16: case XTG_INT32: case XTG_INT64: kind = 'i'; break;
        case XTG_UINT8: case XTG_UINT16: case XTG_UINT32: case XTG_UINT64: kind = 'u'; break;
        case XTG_FLOAT32: case XTG_FLOAT64: kind = 'f'; break;
        default: return std::string();
    }
    const int size = dt(dtype).size;
    std::string s;
    s += size <= 1 ? '|' : (host_little_endian() ? '<' : '>');
    s += kind;
    s += std::to_string(size);
    return s;
}

int dtype_of_typestring(const std::string& d) {
    for (int t = 0; t < XTG_NUM_DTYPES; ++t)
        if (!typestring(t).empty() && typestring(t) == d) return t;
    return -1;
}

// ---- header parsing (the reference's parse_header, xnpy.hpp:237-390) --------
xtg_status unwrap(std::string& s, char front, char back) {
    if (s.size() >= 2 && s.front() == front && s.back() == back) {
        s = s.substr(1, s.size() - 2);
        return XTG_OK;
    }
    return fail(XTG_ERR_INVALID, "unable to unwrap");
}

std::string value_of(std::string kv) {
    if (!kv.empty() && kv.back() == ',') kv.pop_back();
    const size_t c = kv.find(':');
    return c == std::string::npos ? std::string() : kv.substr(c + 1);
}

// '([<>|])([ifucb])(\d+)' matched against the whole quoted value.
bool valid_typestring(const std::string& v) {
    if (v.size() < 5 || v.front() != '\'' || v.back() != '\'') return false;
    if (!strchr("<>|", v[1]) || !strchr("ifucb", v[2])) return false;
    for (size_t i = 3; i + 1 < v.size(); ++i)
        if (v[i] < '0' || v[i] > '9') return false;
    return true;
}

xtg_status parse_header(std::string header, xtg_npy_header* h) {
    if (header.empty() || header.back() != '\n') return fail(XTG_ERR_INVALID, "invalid header");
    header.pop_back();
    header.erase(std::remove(header.begin(), header.end(), ' '), header.end());
    XTG_TRY(unwrap(header, '{', '}'));
    const size_t kd = header.find("'descr'");
    const size_t kf = header.find("'fortran_order'");
    const size_t ks = header.find("'shape'");
    if (kd == std::string::npos) return fail(XTG_ERR_INVALID, "missing 'descr' key");
    if (kf == std::string::npos) return fail(XTG_ERR_INVALID, "missing 'fortran_order' key");
    if (ks == std::string::npos) return fail(XTG_ERR_INVALID, "missing 'shape' key");
    if (kd >= kf || kf >= ks) return fail(XTG_ERR_INVALID, "header keys in wrong order");
    const std::string descr = value_of(header.substr(kd, kf - kd));
    const std::string fortran = value_of(header.substr(kf, ks - kf));
    std::string shape = value_of(header.substr(ks));
    if (!valid_typestring(descr)) return fail(XTG_ERR_INVALID, "invalid typestring");
    const std::string d = descr.substr(1, descr.size() - 2);
    if (d.size() >= sizeof(h->descr)) return fail(XTG_ERR_INVALID, "invalid typestring");
    memset(h->descr, 0, sizeof(h->descr));
    memcpy(h->descr, d.data(), d.size());
    h->dtype = dtype_of_typestring(d);
    if (fortran == "True") h->fortran_order = 1;
    else if (fortran == "False") h->fortran_order = 0;
    else return fail(XTG_ERR_INVALID, "invalid fortran_order value");
    XTG_TRY(unwrap(shape, '(', ')'));
    // "3,3,3" / "5," / "": a comma-separated list, one trailing comma allowed
    std::vector<int64_t> dims;
    size_t pos = 0;
    for (;;) {
        const size_t next = shape.find(',', pos);
        const std::string tok = shape.substr(pos, next == std::string::npos ? std::string::npos : next - pos);
        if (tok.empty()) {
            if (next != std::string::npos) return fail(XTG_ERR_INVALID, "invalid shape");
        } else {
            int64_t v = 0;
            for (char c : tok) {
                if (c < '0' || c > '9' || v > (int64_t(1) << 50)) return fail(XTG_ERR_INVALID, "invalid shape");
                v = v * 10 + (c - '0');
            }
            dims.push_back(v);
        }
        if (next == std::string::npos) break;
        pos = next + 1;
    }
    if ((int)dims.size() > XTG_MAX_RANK)
        return fail(XTG_ERR_UNSUPPORTED, "npy file rank " + std::to_string(dims.size()) + " exceeds XTG_MAX_RANK");
    h->rank = (int)dims.size();
    int64_t n = 1;
    for (int i = 0; i < h->rank; ++i) {
        h->shape[i] = dims[i];
        if (dims[i] != 0 && n > (int64_t(1) << 56) / dims[i]) return fail(XTG_ERR_INVALID, "invalid shape");
        n *= dims[i];
    }
    int64_t item = 0;
    for (size_t i = 2; i < d.size(); ++i) item = item * 10 + (d[i] - '0');
    h->data_bytes = n * item;
    return XTG_OK;
}

// ---- byte sources and sinks ---------------------------------------------------
struct Src {
    int fd = -1;                       // a file …
    const unsigned char* mem = nullptr;  // … or a host buffer
    size_t mem_len = 0;
    bool mem_pinned = false;
    xtg_status read(void* dst, size_t off, size_t len) const {
        if (fd < 0) {
            if (off + len > mem_len) return fail(XTG_ERR_INVALID, "io error: failed reading file");
            memcpy(dst, mem + off, len);
            return XTG_OK;
        }
        unsigned char* p = (unsigned char*)dst;
        while (len) {
            const ssize_t r = pread(fd, p, len, (off_t)off);
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) return fail(XTG_ERR_INVALID, "io error: failed reading file");
            p += r;
            off += (size_t)r;
            len -= (size_t)r;
        }
        return XTG_OK;
    }
};
struct Sink {
    int fd = -1;
    unsigned char* mem = nullptr;
    xtg_status write(const void* src, size_t off, size_t len) const {
        if (fd < 0) {
            memcpy(mem + off, src, len);
            return XTG_OK;
        }
        const unsigned char* p = (const unsigned char*)src;
        while (len) {
            const ssize_t r = pwrite(fd, p, len, (off_t)off);
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) return fail(XTG_ERR_INVALID, "IO Error: failed to write file");
            p += r;
            off += (size_t)r;
            len -= (size_t)r;
        }
        return XTG_OK;
    }
};

struct FdGuard {
    int fd = -1;
    ~FdGuard() {
        if (fd >= 0) close(fd);
    }
};

xtg_status read_header(const Src& src, xtg_npy_header* h) {
    memset(h, 0, sizeof *h);
    unsigned char pre[kMagicLen + 2];
    XTG_TRY(src.read(pre, 0, sizeof pre));
    if (memcmp(pre, kMagic, kMagicLen) != 0) return fail(XTG_ERR_INVALID, "this file do not have a valid npy format.");
    const int major = pre[kMagicLen], minor = pre[kMagicLen + 1];
    size_t lenbytes;
    if (major == 1 && minor == 0) lenbytes = 2;
    else if (major == 2 && minor == 0) lenbytes = 4;
    else return fail(XTG_ERR_INVALID, "unsupported file format version");
    h->version = major;
    unsigned char lb[4] = {0, 0, 0, 0};
    XTG_TRY(src.read(lb, sizeof pre, lenbytes));
    const size_t hlen = (size_t)lb[0] | (size_t)lb[1] << 8 | (size_t)lb[2] << 16 | (size_t)lb[3] << 24;
    const size_t start = sizeof pre + lenbytes;
    std::string header(hlen, '\0');
    if (hlen) XTG_TRY(src.read(&header[0], start, hlen));
    XTG_TRY(parse_header(header, h));
    h->data_offset = (int64_t)(start + hlen);
    return XTG_OK;
}

// The reference's write_header (xnpy.hpp:394-463), byte for byte.
std::string make_header(const std::string& descr, bool fortran, const int64_t* shape, int rank) {
    std::string s_shape = "(";
    for (int i = 0; i < rank; ++i) s_shape += std::to_string(shape[i]) + ", ";
    if (rank > 1) s_shape.erase(s_shape.size() - 2);
    else if (rank == 1) s_shape.erase(s_shape.size() - 1);
    s_shape += ")";
    std::string dict = "{'descr': '" + descr + "', 'fortran_order': " + (fortran ? "True" : "False") +
                       ", 'shape': " + s_shape + ", }";
    const size_t pre_len = dict.size() + 1;
    size_t meta = kMagicLen + 2 + 2 + pre_len;
    unsigned char ver = 1;
    if (meta >= 255 * 255) {
        meta = kMagicLen + 2 + 4 + pre_len;
        ver = 2;
    }
    dict.append(64 - meta % 64, ' ');
    dict += '\n';
    std::string out(kMagic, kMagicLen);
    out += (char)ver;
    out += (char)0;
    const size_t hl = dict.size();
    out += (char)(hl & 0xff);
    out += (char)((hl >> 8) & 0xff);
    if (ver == 2) {
        out += (char)((hl >> 16) & 0xff);
        out += (char)((hl >> 24) & 0xff);
    }
    return out + dict;
}

// ---- staging ring ----------------------------------------------------------------
struct Worker {
    cudaStream_t s = nullptr;
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
};
struct Staging {
    std::mutex mu;  // one npy transfer at a time owns the ring
    int device = -1;
    size_t chunk = 0;
    std::vector<Worker> w;
};
Staging& staging() {
    static Staging* s = new Staging();  // lives for the process: pinned memory outlives static destructors
    return *s;
}

xtg_status staging_ready(Staging& st, int device, int want_workers, size_t chunk) {
    if (st.device == device && st.chunk == chunk && (int)st.w.size() >= want_workers) return XTG_OK;
    if (st.device != device || st.chunk != chunk) {
        for (Worker& w : st.w) {
            for (int b = 0; b < 2; ++b) {
                if (w.buf[b]) cudaFreeHost(w.buf[b]);
                if (w.ev[b]) cudaEventDestroy(w.ev[b]);
            }
            if (w.s) cudaStreamDestroy(w.s);
        }
        st.w.clear();
    }
    st.device = device;
    st.chunk = chunk;
    while ((int)st.w.size() < want_workers) {
        Worker w;
        XTG_CUDA(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking));
        st.w.push_back(w);
        Worker& x = st.w.back();
        for (int b = 0; b < 2; ++b) {
            XTG_CUDA(cudaHostAlloc(&x.buf[b], chunk, cudaHostAllocDefault));
            XTG_CUDA(cudaEventCreateWithFlags(&x.ev[b], cudaEventDisableTiming));
        }
    }
    return XTG_OK;
}

struct Job {
    bool to_device;          // load: src -> dev; save: dev -> sink
    int max_workers = 1 << 30;
    const Src* src = nullptr;
    const Sink* sink = nullptr;
    size_t file_off = 0;     // byte offset of the data in the file / buffer
    unsigned char* dev = nullptr;
    size_t bytes = 0;
    size_t chunk = 0;
    int nworkers = 1;
    int device = 0;
    cudaEvent_t after = nullptr;  // the copies start after this event
    cudaEvent_t wait_for = nullptr;  // if set: the event to start after (else the caller's stream now)
    std::atomic<int> status{XTG_OK};
    std::string msg;
    std::mutex msg_mu;
};

void record_failure(Job& j, xtg_status s) {
    int expect = XTG_OK;
    if (j.status.compare_exchange_strong(expect, (int)s)) {
        std::lock_guard<std::mutex> g(j.msg_mu);
        j.msg = xtg_last_error();
    }
}

#define JOB_TRY(call)                     \
    do {                                  \
        xtg_status _s = (call);           \
        if (_s != XTG_OK) {               \
            record_failure(j, _s);        \
            goto done;                    \
        }                                 \
    } while (0)
#define JOB_CUDA(call)                           \
    do {                                         \
        cudaError_t _e = (call);                 \
        if (_e != cudaSuccess) {                 \
            record_failure(j, cuda_fail(_e, #call)); \
            goto done;                           \
        }                                        \
    } while (0)

void run_worker(Job& j, Worker& w, int wi) {
    const size_t nchunks = (j.bytes + j.chunk - 1) / j.chunk;
    bool pending[2] = {false, false};
    size_t prev_off = 0, prev_len = 0;
    int k = 0;
    if (cudaSetDevice(j.device) != cudaSuccess) {
        record_failure(j, fail(XTG_ERR_CUDA, "cudaSetDevice failed on an npy worker thread"));
        return;
    }
    JOB_CUDA(cudaStreamWaitEvent(w.s, j.after, 0));
    for (size_t c = (size_t)wi; c < nchunks; c += (size_t)j.nworkers, ++k) {
        if (j.status.load(std::memory_order_relaxed) != XTG_OK) break;
        const int b = k & 1;
        const size_t off = c * j.chunk;
        const size_t len = std::min(j.chunk, j.bytes - off);
        if (j.to_device) {
            if (pending[b]) JOB_CUDA(cudaEventSynchronize(w.ev[b]));
            JOB_TRY(j.src->read(w.buf[b], j.file_off + off, len));
            JOB_CUDA(cudaMemcpyAsync(j.dev + off, w.buf[b], len, cudaMemcpyHostToDevice, w.s));
            JOB_CUDA(cudaEventRecord(w.ev[b], w.s));
            pending[b] = true;
        } else {
            JOB_CUDA(cudaMemcpyAsync(w.buf[b], j.dev + off, len, cudaMemcpyDeviceToHost, w.s));
            JOB_CUDA(cudaEventRecord(w.ev[b], w.s));
            if (k > 0) {
                JOB_CUDA(cudaEventSynchronize(w.ev[b ^ 1]));
                JOB_TRY(j.sink->write(w.buf[b ^ 1], j.file_off + prev_off, prev_len));
            }
            prev_off = off;
            prev_len = len;
        }
    }
    if (!j.to_device && k > 0 && j.status.load() == XTG_OK) {
        const int b = (k - 1) & 1;
        JOB_CUDA(cudaEventSynchronize(w.ev[b]));
        JOB_TRY(j.sink->write(w.buf[b], j.file_off + prev_off, prev_len));
    }
done:
    cudaStreamSynchronize(w.s);  // nothing of this call stays in flight on the buffers
}

// Moves j.bytes between the device and the source / sink.  Blocks until
// every chunk has landed; the caller's stream is ordered before the copies.
xtg_status run_job(Job& j, cudaStream_t stream) {
    if (j.bytes == 0) return XTG_OK;
    DeviceInfo* info;
    XTG_TRY(ensure_device(&info));
    j.device = info->device;
    // 4 MiB chunks on up to 16 threads: measured on the GB300's Grace host,
    // loads from the page cache ran 74 GB/s with 8 threads and 89 with 16
    const size_t chunk = (size_t)std::max<int64_t>(opt("npy.chunk_bytes", 4 << 20), 1 << 16) & ~(size_t)4095;
    int nw = (int)opt("npy.threads", std::min(16u, std::max(1u, std::thread::hardware_concurrency())));
    nw = std::max(1, std::min<int>(std::min(nw, j.max_workers), (int)((j.bytes + chunk - 1) / chunk)));
    Staging& st = staging();
    std::lock_guard<std::mutex> g(st.mu);
    XTG_TRY(staging_ready(st, j.device, nw, chunk));
    j.chunk = chunk;
    j.nworkers = nw;
    cudaEvent_t after;
    XTG_CUDA(cudaEventCreateWithFlags(&after, cudaEventDisableTiming));
    j.after = j.wait_for ? j.wait_for : after;
    cudaError_t e = j.wait_for ? cudaSuccess : cudaEventRecord(after, stream);
    if (e == cudaSuccess) {
        std::vector<std::thread> th;
        for (int i = 1; i < nw; ++i) th.emplace_back(run_worker, std::ref(j), std::ref(st.w[i]), i);
        run_worker(j, st.w[0], 0);
        for (auto& t : th) t.join();
    }
    cudaEventDestroy(after);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    if (j.status.load() != XTG_OK) return fail((xtg_status)j.status.load(), j.msg);
    return XTG_OK;
}

// ---- layouts ------------------------------------------------------------------
bool dense_with(const xtg_array& a, bool fortran) {
    int64_t expect = 1;
    for (int k = 0; k < a.rank; ++k) {
        const int d = fortran ? k : a.rank - 1 - k;
        if (a.shape[d] != 1 && a.strides[d] != expect) return false;
        expect *= a.shape[d];
    }
    return true;
}
int64_t numel(const xtg_array& a) {
    int64_t n = 1;
    for (int k = 0; k < a.rank; ++k) n *= a.shape[k];
    return n;
}

xtg_status check_array(const xtg_array* a, const char* what) {
    if (!a) return fail(XTG_ERR_INVALID, std::string("null ") + what);
    if (!valid_dtype(a->dtype)) return fail(XTG_ERR_INVALID, std::string("bad dtype of ") + what);
    if (a->rank < 0 || a->rank > XTG_MAX_RANK) return fail(XTG_ERR_INVALID, std::string("bad rank of ") + what);
    for (int k = 0; k < a->rank; ++k)
        if (a->shape[k] < 0) return fail(XTG_ERR_INVALID, std::string("negative extent in ") + what);
    if (!a->data && numel(*a) > 0) return fail(XTG_ERR_INVALID, std::string("null data of ") + what);
    return XTG_OK;
}

// The data pointer of an array the ring copies to / from must be live device
// memory: a freed or host pointer passed with an explicit copy direction
// would otherwise be dereferenced as host memory.
xtg_status check_device_ptr(const xtg_array& a, const char* what) {
    if (numel(a) == 0 || dry_run()) return XTG_OK;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, a.data) != cudaSuccess) {
        cudaGetLastError();
        return fail(XTG_ERR_INVALID, std::string(what) + " is not device memory");
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
        return fail(XTG_ERR_INVALID, std::string(what) + " is not device memory");
    return XTG_OK;
}

xtg_status assign_copy(const xtg_array& from, const xtg_array& to, cudaStream_t stream) {
    xtg_expr e;
    memset(&e, 0, sizeof e);
    e.n_nodes = 1;
    e.n_leaves = 1;
    e.leaves[0] = from;
    e.nodes[0].op = XTG_OP_LEAF;
    e.nodes[0].dtype = from.dtype;
    e.nodes[0].arg = 0;
    return xtg_assign(&e, &to, stream);
}

xtg_status load_impl(const Src& src, const xtg_array* out, int32_t layout, cudaStream_t stream) {
    XTG_TRY(check_array(out, "destination"));
    XTG_TRY(check_device_ptr(*out, "destination"));
    xtg_npy_header h;
    XTG_TRY(read_header(src, &h));
    const std::string want = typestring(out->dtype);
    if (want.empty()) return fail(XTG_ERR_UNSUPPORTED, std::string("no npy typestring for ") + dt(out->dtype).cname);
    if (want != h.descr)
        return fail(XTG_ERR_INVALID, std::string("Cast error: formats not matching ") + h.descr + " vs " + want);
    if ((layout == XTG_LAYOUT_COLUMN_MAJOR && !h.fortran_order) || (layout == XTG_LAYOUT_ROW_MAJOR && h.fortran_order))
        return fail(XTG_ERR_INVALID, "Cast error: layout mismatch between npy file and requested layout.");
    if (layout < XTG_LAYOUT_DYNAMIC || layout > XTG_LAYOUT_COLUMN_MAJOR)
        return fail(XTG_ERR_INVALID, "bad layout");
    bool same = out->rank == h.rank;
    for (int k = 0; same && k < h.rank; ++k) same = out->shape[k] == h.shape[k];
    if (!same) return fail(XTG_ERR_SHAPE, "npy file shape does not match the destination");
    if (src.fd < 0 && (size_t)(h.data_offset + h.data_bytes) > src.mem_len)
        return fail(XTG_ERR_INVALID, "io error: failed reading file");
    if (h.data_bytes == 0) return XTG_OK;

    xtg_array file_arr = *out;  // the file's elements, as a strided array of its order
    {
        int64_t s = 1;
        for (int k = 0; k < h.rank; ++k) {
            const int d = h.fortran_order ? k : h.rank - 1 - k;
            file_arr.strides[d] = s;
            s *= h.shape[d];
        }
    }
    const bool direct = dense_with(*out, h.fortran_order != 0);
    void* tmp = nullptr;
    if (!direct) {
        XTG_TRY(scratch_alloc(&tmp, (size_t)h.data_bytes, stream));
        file_arr.data = tmp;
    }
    Job j;
    j.to_device = true;
    j.src = &src;
    j.file_off = (size_t)h.data_offset;
    j.dev = (unsigned char*)(direct ? out->data : tmp);
    j.bytes = (size_t)h.data_bytes;
    xtg_status s;
    if (src.fd < 0 && src.mem_pinned) {
        // page-locked buffer: one DMA straight from it
        cudaError_t e = cudaMemcpyAsync(j.dev, src.mem + j.file_off, j.bytes, cudaMemcpyHostToDevice, stream);
        s = e == cudaSuccess ? XTG_OK : cuda_fail(e, "cudaMemcpyAsync");
        if (s == XTG_OK) {
            e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) s = cuda_fail(e, "cudaStreamSynchronize");
        }
    } else {
        s = run_job(j, stream);
    }
    if (s == XTG_OK && !direct) s = assign_copy(file_arr, *out, stream);
    if (tmp) {
        xtg_status f = scratch_free(tmp, stream);
        if (s == XTG_OK) s = f;
    }
    return s;
}

// The file image's header and where its data comes from on the device.
struct SavePlan {
    std::string header;
    xtg_array src;       // dense device array whose bytes are the data
    void* tmp = nullptr;
    size_t bytes = 0;
};

xtg_status save_prepare(const xtg_array* in, cudaStream_t stream, SavePlan* p) {
    XTG_TRY(check_array(in, "source"));
    XTG_TRY(check_device_ptr(*in, "source"));
    const std::string ts = typestring(in->dtype);
    if (ts.empty()) return fail(XTG_ERR_UNSUPPORTED, std::string("no npy typestring for ") + dt(in->dtype).cname);
    const bool c = numel(*in) == 0 || dense_with(*in, false);
    const bool f = !c && in->rank > 1 && dense_with(*in, true);
    p->header = make_header(ts, f, in->shape, in->rank);
    p->bytes = (size_t)(numel(*in) * dt(in->dtype).size);
    p->src = *in;
    if (!c && !f && p->bytes) {
        XTG_TRY(scratch_alloc(&p->tmp, p->bytes, stream));
        xtg_array t = *in;
        t.data = p->tmp;
        int64_t s = 1;
        for (int k = in->rank - 1; k >= 0; --k) {
            t.strides[k] = s;
            s *= in->shape[k];
        }
        xtg_status st = assign_copy(*in, t, stream);
        if (st != XTG_OK) {
            scratch_free(p->tmp, stream);
            p->tmp = nullptr;
            return st;
        }
        p->src = t;
    }
    return XTG_OK;
}

xtg_status save_run(SavePlan& p, const Sink& sink_in, cudaStream_t stream) {
    Job j;
    j.to_device = false;
    j.file_off = p.header.size();
    j.dev = (unsigned char*)p.src.data;
    j.bytes = p.bytes;
    Sink sink = sink_in;
    void* map = nullptr;
    const size_t total = p.header.size() + p.bytes;
    if (sink.fd >= 0) {
        struct statfs fs;
        const bool tmpfs = fstatfs(sink.fd, &fs) == 0 && (unsigned long)fs.f_type == 0x01021994UL;
        if (tmpfs && p.bytes >= ((size_t)1 << 20)) {
            // the pages are allocated up front, so no store into the mapping
            // can meet a full file system (that would be a SIGBUS, not an error)
            if (fallocate(sink.fd, 0, 0, (off_t)total) != 0) {
                if (p.tmp) scratch_free(p.tmp, stream);
                p.tmp = nullptr;
                return fail(XTG_ERR_INVALID, std::string("IO Error: failed to write file: ") + strerror(errno));
            }
            map = mmap(nullptr, total, PROT_READ | PROT_WRITE, MAP_SHARED, sink.fd, 0);
            if (map == MAP_FAILED) map = nullptr;
        }
        if (map) {
            sink.fd = -1;
            sink.mem = (unsigned char*)map;
        } else {
            j.max_workers = 1;  // writes in file order from one thread
            if (p.bytes) (void)fallocate(sink.fd, 0, 0, (off_t)total);  // no emulation where unsupported
        }
    }
    j.sink = &sink;
    xtg_status s = sink.write(p.header.data(), 0, p.header.size());
    if (s == XTG_OK) s = run_job(j, stream);
    if (map && munmap(map, total) != 0 && s == XTG_OK) s = fail(XTG_ERR_INVALID, "IO Error: failed to write file");
    if (p.tmp) {
        xtg_status f = scratch_free(p.tmp, stream);
        if (s == XTG_OK) s = f;
        p.tmp = nullptr;
    }
    return s;
}

bool host_pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

}  // namespace

xtg_status ring_h2d(void* dev, const void* host, size_t bytes, cudaEvent_t wait_for) {
    Src src;
    src.mem = (const unsigned char*)host;
    src.mem_len = bytes;
    Job j;
    j.to_device = true;
    j.src = &src;
    j.dev = (unsigned char*)dev;
    j.bytes = bytes;
    j.wait_for = wait_for;
    return run_job(j, nullptr);
}

}  // namespace xtgh

using namespace xtgh;

extern "C" xtg_status xtg_npy_info(const char* path, xtg_npy_header* h) {
    clear_error();
    if (!path || !h) return fail(XTG_ERR_INVALID, "null argument");
    FdGuard fd;
    fd.fd = open(path, O_RDONLY | O_CLOEXEC);
    if (fd.fd < 0) return fail(XTG_ERR_INVALID, "io error: failed to open a file.");
    Src src;
    src.fd = fd.fd;
    return read_header(src, h);
}

extern "C" xtg_status xtg_npy_info_buffer(const void* buf, size_t len, xtg_npy_header* h) {
    clear_error();
    if ((!buf && len) || !h) return fail(XTG_ERR_INVALID, "null argument");
    Src src;
    src.mem = (const unsigned char*)buf;
    src.mem_len = len;
    return read_header(src, h);
}

extern "C" xtg_status xtg_npy_format_header(int32_t dtype, int32_t fortran_order, int32_t rank, const int64_t* shape,
                                            char* buf, size_t cap, size_t* len) {
    clear_error();
    if (!len || (rank > 0 && !shape)) return fail(XTG_ERR_INVALID, "null argument");
    if (!valid_dtype(dtype)) return fail(XTG_ERR_INVALID, "bad dtype");
    if (rank < 0 || rank > XTG_MAX_RANK) return fail(XTG_ERR_INVALID, "bad rank");
    const std::string ts = typestring(dtype);
    if (ts.empty()) return fail(XTG_ERR_UNSUPPORTED, std::string("no npy typestring for ") + dt(dtype).cname);
    const std::string h = make_header(ts, fortran_order != 0, shape, rank);
    *len = h.size();
    if (!buf) return XTG_OK;
    if (cap < h.size()) return fail(XTG_ERR_INVALID, "npy buffer too small");
    memcpy(buf, h.data(), h.size());
    return XTG_OK;
}

extern "C" xtg_status xtg_npy_load(const char* path, const xtg_array* out, int32_t layout, xtg_stream stream) {
    clear_error();
    begin_call();
    if (!path) return fail(XTG_ERR_INVALID, "null path");
    FdGuard fd;
    fd.fd = open(path, O_RDONLY | O_CLOEXEC);
    if (fd.fd < 0) return fail(XTG_ERR_INVALID, "io error: failed to open a file.");
    Src src;
    src.fd = fd.fd;
    return load_impl(src, out, layout, (cudaStream_t)stream);
}

extern "C" xtg_status xtg_npy_load_buffer(const void* buf, size_t len, const xtg_array* out, int32_t layout,
                                          xtg_stream stream) {
    clear_error();
    begin_call();
    if (!buf && len) return fail(XTG_ERR_INVALID, "null buffer");
    Src src;
    src.mem = (const unsigned char*)buf;
    src.mem_len = len;
    src.mem_pinned = buf && !dry_run() && host_pinned(buf);
    return load_impl(src, out, layout, (cudaStream_t)stream);
}

extern "C" xtg_status xtg_npy_save(const char* path, const xtg_array* in, xtg_stream stream) {
    clear_error();
    begin_call();
    if (!path) return fail(XTG_ERR_INVALID, "null path");
    SavePlan p;
    XTG_TRY(save_prepare(in, (cudaStream_t)stream, &p));
    FdGuard fd;
    fd.fd = open(path, O_RDWR | O_CREAT | O_TRUNC | O_CLOEXEC, 0644);
    if (fd.fd < 0) {
        if (p.tmp) scratch_free(p.tmp, (cudaStream_t)stream);
        return fail(XTG_ERR_INVALID, std::string("IO Error: failed to open file: ") + path);
    }
    Sink sink;
    sink.fd = fd.fd;
    return save_run(p, sink, (cudaStream_t)stream);
}

extern "C" xtg_status xtg_npy_save_buffer(const xtg_array* in, void* buf, size_t cap, size_t* len,
                                          xtg_stream stream) {
    clear_error();
    begin_call();
    if (!len) return fail(XTG_ERR_INVALID, "null length");
    XTG_TRY(check_array(in, "source"));
    const std::string ts = typestring(in->dtype);
    if (ts.empty()) return fail(XTG_ERR_UNSUPPORTED, std::string("no npy typestring for ") + dt(in->dtype).cname);
    const bool c = numel(*in) == 0 || dense_with(*in, false);
    const bool f = !c && in->rank > 1 && dense_with(*in, true);
    const size_t total = make_header(ts, f, in->shape, in->rank).size() + (size_t)(numel(*in) * dt(in->dtype).size);
    *len = total;
    if (!buf) return XTG_OK;
    if (cap < total) return fail(XTG_ERR_INVALID, "npy buffer too small");
    SavePlan p;
    XTG_TRY(save_prepare(in, (cudaStream_t)stream, &p));
    if (p.bytes && host_pinned(buf)) {
        memcpy(buf, p.header.data(), p.header.size());
        xtg_status s = XTG_OK;
        cudaError_t e = cudaMemcpyAsync((unsigned char*)buf + p.header.size(), p.src.data, p.bytes,
                                        cudaMemcpyDeviceToHost, (cudaStream_t)stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess) s = cuda_fail(e, "npy copy to a pinned buffer");
        if (p.tmp) {
            xtg_status fs = scratch_free(p.tmp, (cudaStream_t)stream);
            if (s == XTG_OK) s = fs;
        }
        return s;
    }
    Sink sink;
    sink.mem = (unsigned char*)buf;
    return save_run(p, sink, (cudaStream_t)stream);
}
