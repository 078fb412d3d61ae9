/*
 * pm_io.cpp — the reference's image files for real stereo pairs (host code).
 *
 *   CVTRaw  plugins/iloader/CVTRaw/CVTRawLoader.cpp, plugins/isaver/CVTRaw/CVTRawSaver.cpp
 *   PPM/PGM plugins/iloader/PPM/PPMLoader.cpp
 *   PFM     plugins/isaver/PFM/PFMSaver.cpp
 *
 * Readers work in two calls on one cvtpm_image descriptor: with data == NULL
 * they fill format, width, height and a tight stride; with data set they read
 * the pixels.  Errors are reported through the status and the thread's
 * context-free error message (cvtpm_last_error(NULL)).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "cvtpm.h"

void pm_set_free_error(const std::string& m);   /* pm_image.cu */

namespace {

cvtpm_status fail(cvtpm_status s, const std::string& m) {
    pm_set_free_error(m);
    return s;
}

/* a host allocation sized by the file or image failed: no exception leaves
 * the C ABI */
cvtpm_status pm_out_of_memory() { return fail(CVTPM_ERR_ALLOC, "host memory exhausted"); }

bool read_file(const char* path, std::vector<unsigned char>* out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    out->clear();
    unsigned char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out->insert(out->end(), buf, buf + n);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

bool little_endian() {
    const uint16_t v = 1;
    unsigned char b;
    memcpy(&b, &v, 1);
    return b == 1;
}

/* netpbm header tokens: whitespace separated, '#' starts a comment to the end
 * of the line.  Returns false at the end of the data. */
bool next_token(const std::vector<unsigned char>& d, size_t* pos, std::string* tok) {
    size_t i = *pos;
    for (;;) {
        while (i < d.size() && (d[i] == ' ' || d[i] == '\t' || d[i] == '\n' || d[i] == '\r')) ++i;
        if (i < d.size() && d[i] == '#') {
            while (i < d.size() && d[i] != '\n') ++i;
            continue;
        }
        break;
    }
    if (i >= d.size()) return false;
    const size_t b = i;
    while (i < d.size() && !(d[i] == ' ' || d[i] == '\t' || d[i] == '\n' || d[i] == '\r' || d[i] == '#')) ++i;
    tok->assign((const char*)&d[b], i - b);
    *pos = i;
    return true;
}

bool to_int(const std::string& t, long* v) {
    if (t.empty()) return false;
    char* e = nullptr;
    *v = strtol(t.c_str(), &e, 10);
    return e && *e == '\0';
}

}  // namespace

extern "C" {

static cvtpm_status cvtpm_raw_read_impl(const char* path, cvtpm_image* img) {
    if (!path || !img) return fail(CVTPM_ERR_INVALID_ARGUMENT, "raw read: path or descriptor is NULL");
    std::vector<unsigned char> d;
    if (!read_file(path, &d)) return fail(CVTPM_ERR_IO, std::string("raw read: cannot read ") + path);
    if (d.size() < 16) return fail(CVTPM_ERR_IO, "raw read: header truncated");
    uint32_t h[4];   /* width, height, stride, IFormatID (CVTRawLoader.cpp) */
    memcpy(h, d.data(), 16);
    const size_t bpp = cvtpm_iformat_bpp((int)h[3]);
    if (!bpp) return fail(CVTPM_ERR_IO, "raw read: unknown format id " + std::to_string(h[3]));
    if (h[0] == 0 || h[1] == 0 || h[0] > (1u << 30) / bpp || h[1] > (1u << 30))
        return fail(CVTPM_ERR_IO, "raw read: bad size");
    const size_t row = (size_t)h[0] * bpp;
    if (h[2] < row) return fail(CVTPM_ERR_IO, "raw read: stored stride below width * bytes per pixel");
    if (d.size() - 16 < (size_t)h[2] * (h[1] - 1) + row) return fail(CVTPM_ERR_IO, "raw read: pixel data truncated");
    if (!img->data) {
        img->format = (int)h[3];
        img->width = (int)h[0];
        img->height = (int)h[1];
        img->stride = row;
        return CVTPM_OK;
    }
    if (img->format != (int)h[3] || img->width != (int)h[0] || img->height != (int)h[1] || img->stride < row)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "raw read: descriptor does not match the file");
    for (uint32_t y = 0; y < h[1]; ++y)
        memcpy((unsigned char*)img->data + (size_t)y * img->stride, d.data() + 16 + (size_t)y * h[2], row);
    return CVTPM_OK;
}

cvtpm_status cvtpm_raw_read(const char* path, cvtpm_image* img) {
    try {
        return cvtpm_raw_read_impl(path, img);
    } catch (const std::bad_alloc&) {
        return pm_out_of_memory();
    }
}

static cvtpm_status cvtpm_raw_write_impl(const char* path, const cvtpm_image* img) {
    if (!path || !img || !img->data) return fail(CVTPM_ERR_INVALID_ARGUMENT, "raw write: NULL argument");
    const size_t bpp = cvtpm_iformat_bpp(img->format);
    if (!bpp) return fail(CVTPM_ERR_INVALID_ARGUMENT, "raw write: unknown format");
    if (img->width < 1 || img->height < 1 || img->stride < (size_t)img->width * bpp || img->stride > 0xffffffffu)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "raw write: bad size or stride");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(CVTPM_ERR_IO, std::string("raw write: cannot open ") + path);
    /* the saver writes the image's own stride and every row in full */
    const uint32_t h[4] = {(uint32_t)img->width, (uint32_t)img->height, (uint32_t)img->stride, (uint32_t)img->format};
    bool ok = fwrite(h, 4, 4, f) == 4 &&
              fwrite(img->data, 1, img->stride * (size_t)img->height, f) == img->stride * (size_t)img->height;
    ok = (fclose(f) == 0) && ok;
    return ok ? CVTPM_OK : fail(CVTPM_ERR_IO, std::string("raw write: write failed for ") + path);
}

cvtpm_status cvtpm_raw_write(const char* path, const cvtpm_image* img) {
    try {
        return cvtpm_raw_write_impl(path, img);
    } catch (const std::bad_alloc&) {
        return pm_out_of_memory();
    }
}

static cvtpm_status cvtpm_ppm_read_impl(const char* path, cvtpm_image* img) {
    if (!path || !img) return fail(CVTPM_ERR_INVALID_ARGUMENT, "ppm read: path or descriptor is NULL");
    std::vector<unsigned char> d;
    if (!read_file(path, &d)) return fail(CVTPM_ERR_IO, std::string("ppm read: cannot read ") + path);
    size_t pos = 0;
    std::string t;
    if (!next_token(d, &pos, &t)) return fail(CVTPM_ERR_IO, "ppm read: PPM header corrupt");
    int kind;
    if (t == "P2") kind = 2;
    else if (t == "P3") kind = 3;
    else if (t == "P5") kind = 5;
    else if (t == "P6") kind = 6;
    else return fail(CVTPM_ERR_IO, "ppm read: unknown PGM type: " + t);
    long w, h, maxv;
    if (!next_token(d, &pos, &t) || !to_int(t, &w) || !next_token(d, &pos, &t) || !to_int(t, &h))
        return fail(CVTPM_ERR_IO, "ppm read: PPM header corrupt: expected <width> <height>");
    if (!next_token(d, &pos, &t) || !to_int(t, &maxv))
        return fail(CVTPM_ERR_IO, "ppm read: PPM header corrupt: expected <color depth>");
    if (w < 1 || h < 1 || w > (1 << 28) || h > (1 << 28) || maxv < 1)
        return fail(CVTPM_ERR_IO, "ppm read: bad size or colour depth");
    if (maxv > 255) return fail(CVTPM_ERR_NOT_SUPPORTED, "ppm read: colour depth above 255");
    const bool rgb = kind == 3 || kind == 6;
    const int fmt = rgb ? CVTPM_IFORMAT_RGBA_UINT8 : CVTPM_IFORMAT_GRAY_UINT8;
    const size_t row = (size_t)w * (rgb ? 4 : 1);
    if (!img->data) {
        img->format = fmt;
        img->width = (int)w;
        img->height = (int)h;
        img->stride = row;
        return CVTPM_OK;
    }
    if (img->format != fmt || img->width != (int)w || img->height != (int)h || img->stride < row)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "ppm read: descriptor does not match the file");
    const size_t nin = (size_t)w * (rgb ? 3 : 1);
    if (kind == 5 || kind == 6) {
        ++pos;   /* the single whitespace character after the colour depth */
        if (pos > d.size() || d.size() - pos < nin * (size_t)h) return fail(CVTPM_ERR_IO, "ppm read: not enough data");
        for (long y = 0; y < h; ++y) {
            unsigned char* o = (unsigned char*)img->data + (size_t)y * img->stride;
            const unsigned char* s = d.data() + pos + (size_t)y * nin;
            if (rgb) {
                for (long x = 0; x < w; ++x) {
                    o[4 * x] = s[3 * x];
                    o[4 * x + 1] = s[3 * x + 1];
                    o[4 * x + 2] = s[3 * x + 2];
                    o[4 * x + 3] = 255;
                }
            } else {
                memcpy(o, s, nin);
            }
        }
        return CVTPM_OK;
    }
    for (long y = 0; y < h; ++y) {   /* ASCII: values truncated to 8 bits, as the reference's (uint8_t) cast */
        unsigned char* o = (unsigned char*)img->data + (size_t)y * img->stride;
        for (long x = 0; x < w; ++x) {
            for (int c = 0; c < (rgb ? 3 : 1); ++c) {
                long v;
                if (!next_token(d, &pos, &t) || !to_int(t, &v)) return fail(CVTPM_ERR_IO, "ppm read: not enough data");
                o[rgb ? 4 * x + c : x] = (unsigned char)v;
            }
            if (rgb) o[4 * x + 3] = 255;
        }
    }
    return CVTPM_OK;
}

cvtpm_status cvtpm_ppm_read(const char* path, cvtpm_image* img) {
    try {
        return cvtpm_ppm_read_impl(path, img);
    } catch (const std::bad_alloc&) {
        return pm_out_of_memory();
    }
}

static cvtpm_status cvtpm_pfm_write_impl(const char* path, const cvtpm_image* img) {
    if (!path || !img || !img->data) return fail(CVTPM_ERR_INVALID_ARGUMENT, "pfm write: NULL argument");
    int ch;
    if (img->format == CVTPM_IFORMAT_GRAY_FLOAT) ch = 1;
    else if (img->format == CVTPM_IFORMAT_RGBA_FLOAT || img->format == CVTPM_IFORMAT_BGRA_FLOAT) ch = 4;
    else return fail(CVTPM_ERR_NOT_SUPPORTED, "pfm write: only GRAY_FLOAT, RGBA_FLOAT and BGRA_FLOAT");
    if (img->width < 1 || img->height < 1 || img->stride < (size_t)img->width * ch * 4)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "pfm write: bad size or stride");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(CVTPM_ERR_IO, std::string("pfm write: cannot open ") + path);
    bool ok = fprintf(f, "%s\n%d %d\n%s1.0\n", ch == 1 ? "Pf" : "PF", img->width, img->height,
                      little_endian() ? "-" : "") > 0;
    std::vector<float> line((size_t)img->width * (ch == 1 ? 1 : 3));
    for (int y = img->height - 1; ok && y >= 0; --y) {   /* bottom to top */
        const float* r = (const float*)((const unsigned char*)img->data + (size_t)y * img->stride);
        if (ch == 1) {
            memcpy(line.data(), r, line.size() * 4);
        } else {
            for (int x = 0; x < img->width; ++x) {   /* the alpha channel dropped, order kept */
                line[3 * x] = r[4 * x];
                line[3 * x + 1] = r[4 * x + 1];
                line[3 * x + 2] = r[4 * x + 2];
            }
        }
        ok = fwrite(line.data(), 4, line.size(), f) == line.size();
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? CVTPM_OK : fail(CVTPM_ERR_IO, std::string("pfm write: write failed for ") + path);
}

cvtpm_status cvtpm_pfm_write(const char* path, const cvtpm_image* img) {
    try {
        return cvtpm_pfm_write_impl(path, img);
    } catch (const std::bad_alloc&) {
        return pm_out_of_memory();
    }
}

}  // extern "C"
