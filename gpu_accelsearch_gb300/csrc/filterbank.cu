// filterbank.cu -- SIGPROC filterbank reader (accel_read_filterbank), host
// only: the raw-data input of the dedispersion step upstream of the search.
// The reference reads dedispersed .dat series only (bpd_data.c); this reads
// the channelised data that dedispersion turns into them.
//
// Format (SIGPROC): a header of keywords, each an int32 byte count and that
// many characters, between HEADER_START and HEADER_END; a keyword is
// followed by its value (int32, float64 or a counted string, by keyword).
// The keyword "signed" takes a single byte (nonzero: 8-bit samples are
// two's-complement, as some writers mark them).  Then the samples,
// time-major: for every time sample nifs x nchans values of nbits bits (8:
// unsigned, or signed where the header says so; 16: unsigned; 32: float32).  The reader
// returns them channel-major, float32 [nchans][nsamples], the layout
// accel_dedisperse takes; channel c is at fch1 + c * foff MHz.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/accelsearch.h"
#include "accel_internal.h"

namespace {

enum Kind { K_INT, K_DBL, K_STR, K_BYTE, K_NONE };

Kind keyword_kind(const std::string& k) {
    static const char* ints[] = {"telescope_id", "machine_id", "data_type", "barycentric", "pulsarcentric",
                                 "nbits", "nsamples", "nchans", "nifs", "nbeams", "ibeam"};
    static const char* dbls[] = {"az_start", "za_start", "src_raj", "src_dej", "tstart", "tsamp",
                                 "fch1", "foff", "refdm", "period"};
    static const char* strs[] = {"rawdatafile", "source_name"};
    for (const char* s : ints)
        if (k == s) return K_INT;
    for (const char* s : dbls)
        if (k == s) return K_DBL;
    for (const char* s : strs)
        if (k == s) return K_STR;
    if (k == "signed") return K_BYTE;
    return K_NONE;
}

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

bool read_string(FILE* f, std::string* out) {
    int32_t n = 0;
    if (fread(&n, sizeof n, 1, f) != 1 || n < 0 || n > 4096) return false;
    out->assign((size_t)n, '\0');
    return n == 0 || fread(&(*out)[0], 1, (size_t)n, f) == (size_t)n;
}

}  // namespace

extern "C" {

int accel_read_filterbank(const char* path, accel_filterbank_info* info, float** data) {
    if (!path || !info || !data) return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: null argument");
    *data = nullptr;
    std::memset(info, 0, sizeof(*info));
    info->nifs = 1;
    File fb;
    fb.f = fopen(path, "rb");
    if (!fb.f) return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: cannot open %s", path);
    std::string key;
    if (!read_string(fb.f, &key) || key != "HEADER_START")
        return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: %s has no SIGPROC header", path);
    long long nsamples_hdr = -1;
    for (;;) {
        if (!read_string(fb.f, &key))
            return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: truncated header");
        if (key == "HEADER_END") break;
        const Kind kind = keyword_kind(key);
        if (kind == K_INT) {
            int32_t v;
            if (fread(&v, sizeof v, 1, fb.f) != 1)
                return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: truncated header");
            if (key == "nbits") info->nbits = v;
            else if (key == "nchans") info->nchans = v;
            else if (key == "nifs") info->nifs = v;
            else if (key == "nsamples") nsamples_hdr = v;
        } else if (kind == K_DBL) {
            double v;
            if (fread(&v, sizeof v, 1, fb.f) != 1)
                return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: truncated header");
            if (key == "tsamp") info->tsamp = v;
            else if (key == "fch1") info->fch1 = v;
            else if (key == "foff") info->foff = v;
            else if (key == "tstart") info->tstart = v;
        } else if (kind == K_BYTE) {
            unsigned char v;
            if (fread(&v, 1, 1, fb.f) != 1)
                return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: truncated header");
            info->is_signed = v != 0;
        } else if (kind == K_STR) {
            std::string v;
            if (!read_string(fb.f, &v))
                return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: truncated header");
            if (key == "source_name") {
                std::strncpy(info->source_name, v.c_str(), sizeof(info->source_name) - 1);
            }
        } else {
            return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: unknown header keyword '%s'",
                                    key.c_str());
        }
    }
    const long pos = ftell(fb.f);
    info->header_bytes = (int)pos;
    if (info->nchans < 1 || info->nifs != 1 || !(info->tsamp > 0.0))
        return accel::set_error(ACCEL_ERR_UNSUPPORTED,
                                "accel_read_filterbank: need nchans >= 1, nifs = 1 and tsamp > 0");
    if (info->nbits != 8 && info->nbits != 16 && info->nbits != 32)
        return accel::set_error(ACCEL_ERR_UNSUPPORTED, "accel_read_filterbank: %d-bit samples not supported",
                                info->nbits);
    if (fseek(fb.f, 0, SEEK_END) != 0) return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: seek");
    const long long bytes = (long long)ftell(fb.f) - pos;
    const long long row = (long long)info->nchans * (info->nbits / 8);
    long long ns = bytes / row;
    if (nsamples_hdr >= 0 && nsamples_hdr < ns) ns = nsamples_hdr;
    if (ns < 1) return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: no samples");
    info->nsamples = ns;
    if (fseek(fb.f, pos, SEEK_SET) != 0) return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: seek");
    float* out = (float*)malloc(sizeof(float) * (size_t)ns * (size_t)info->nchans);
    if (!out) return accel::set_error(ACCEL_ERR_NOMEM, "accel_read_filterbank: host memory");
    // time-major blocks of samples, transposed into the channel-major output
    const long long block = 4096;
    std::vector<unsigned char> buf((size_t)(block * row));
    const int nc = info->nchans;
    for (long long t0 = 0; t0 < ns; t0 += block) {
        const long long nt = std::min(block, ns - t0);
        if (fread(buf.data(), 1, (size_t)(nt * row), fb.f) != (size_t)(nt * row)) {
            free(out);
            return accel::set_error(ACCEL_ERR_INVALID, "accel_read_filterbank: truncated data");
        }
        for (long long t = 0; t < nt; t++) {
            const unsigned char* p = buf.data() + t * row;
            for (int c = 0; c < nc; c++) {
                float v;
                if (info->nbits == 8) {
                    v = info->is_signed ? (float)(int)(signed char)p[c] : (float)p[c];
                } else if (info->nbits == 16) {
                    uint16_t u;
                    std::memcpy(&u, p + 2 * c, 2);
                    v = (float)u;
                } else {
                    std::memcpy(&v, p + 4 * c, 4);
                }
                out[(size_t)c * ns + (t0 + t)] = v;
            }
        }
    }
    *data = out;
    return ACCEL_OK;
}

void accel_free_host(void* p) { free(p); }

}  // extern "C"
