// sphmp_io.cpp — particle data formats on either side of the step: the
// reference's text frame dump, its BINX-020 (.bi2) particle-file reader and
// shape import, and this library's binary state checkpoint. Host code only; the
// checkpoint goes through the public transfer functions.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "sphmp.h"

namespace sphmp {
// Record the text returned by sphmp_last_error on the calling thread (sphmp_api.cu).
sphmp_status record_error(sphmp_status st, const char* msg);
}  // namespace sphmp

using namespace sphmp;

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(FILE* p) : f(p) {}
    ~File() {
        if (f) fclose(f);
    }
};

bool host_little_endian() {
    const uint32_t one = 1;
    unsigned char b;
    memcpy(&b, &one, 1);
    return b == 1;
}

void swap32(void* data, size_t count) {
    unsigned char* p = static_cast<unsigned char*>(data);
    for (size_t i = 0; i < count; i++, p += 4) {
        unsigned char t = p[0];
        p[0] = p[3];
        p[3] = t;
        t = p[1];
        p[1] = p[2];
        p[2] = t;
    }
}

bool read_exact(FILE* f, void* dst, size_t bytes) { return fread(dst, 1, bytes, f) == bytes; }

// BINX-020 layout (SPH_Solver/catpaw/BI2Reader.h:38-58): a 20-byte format head
// (16-char title, fmt, bitorder 1 = big endian, full, data2d), then either the
// 52-byte full data head (h, dp, b, rhop0, gamma, massbound, massfluid, np,
// nfixed, nmoving, nfloat, nfluidout, timestep) or the 24-byte short one (np,
// nfixed, nmoving, nfloat, nfluidout, timestep), every field 4 bytes.
struct Bi2Head {
    char titu[16];
    unsigned char fmt, bitorder, full, data2d;
};

}  // namespace

extern "C" {

sphmp_status sphmp_write_frame_text(const char* path, const sphmp_display_pack* disp, const sphmp_calc_pack* calc,
                                    int32_t n) {
    if (!path || n < 0 || (n > 0 && (!disp || !calc))) return record_error(SPHMP_ERR_INVALID_ARG, "bad arguments");
    File f(fopen(path, "w"));
    if (!f.f) return record_error(SPHMP_ERR_INVALID_ARG, "cannot open the frame file for writing");
    // FluidSystem::outputFile (SPH_Solver/fluids/FluidIOUtility.cpp:17-38)
    fprintf(f.f, "%d\n", n);
    for (int32_t i = 0; i < n; i++) {
        fprintf(f.f, "%f %f %f ", disp[i].pos[0], disp[i].pos[1], disp[i].pos[2]);
        fprintf(f.f, "%f %f %d\n", calc[i].mass, calc[i].restdens, disp[i].type);
    }
    if (ferror(f.f)) return record_error(SPHMP_ERR_INVALID_ARG, "write error on the frame file");
    return SPHMP_OK;
}

sphmp_status sphmp_read_bi2(const char* path, sphmp_bi2_info* info, float* pos, float* vel, float* rhop,
                            int32_t cap) {
    if (!path || !info) return record_error(SPHMP_ERR_INVALID_ARG, "bad arguments");
    memset(info, 0, sizeof(*info));
    File f(fopen(path, "rb"));
    if (!f.f) return record_error(SPHMP_ERR_INVALID_ARG, "cannot open the .bi2 file");
    // BI2Reader::GetInfo(false) (SPH_Solver/catpaw/BI2Reader.cpp:19-106)
    Bi2Head head;
    if (!read_exact(f.f, &head, sizeof(head))) return record_error(SPHMP_ERR_INVALID_ARG, "truncated .bi2 head");
    const bool title = memcmp(head.titu, "#File BINX-020 ", 16) == 0;
    if (!title && head.full > 1)
        return record_error(SPHMP_ERR_INVALID_ARG, "not a BINX-020 particle file");
    const bool swap = (head.bitorder != 0) == host_little_endian();
    info->fmt = 20;
    info->bitorder = head.bitorder;
    info->full = head.full != 0;
    info->data2d = head.data2d != 0;
    if (info->full) {
        float hf[7];
        int32_t hi[5];
        float ts;
        if (!read_exact(f.f, hf, sizeof(hf)) || !read_exact(f.f, hi, sizeof(hi)) || !read_exact(f.f, &ts, 4))
            return record_error(SPHMP_ERR_INVALID_ARG, "truncated .bi2 data head");
        if (swap) {
            swap32(hf, 7);
            swap32(hi, 5);
            swap32(&ts, 1);
        }
        info->h = hf[0];
        info->dp = hf[1];
        info->b = hf[2];
        info->rhop0 = hf[3];
        info->gamma = hf[4];
        info->massbound = hf[5];
        info->massfluid = hf[6];
        info->np = hi[0];
        info->nfixed = hi[1];
        info->nmoving = hi[2];
        info->nfloat = hi[3];
        info->nfluidout = hi[4];
        info->time = ts;
    } else {
        int32_t hi[5];
        float ts;
        if (!read_exact(f.f, hi, sizeof(hi)) || !read_exact(f.f, &ts, 4))
            return record_error(SPHMP_ERR_INVALID_ARG, "truncated .bi2 data head");
        if (swap) {
            swap32(hi, 5);
            swap32(&ts, 1);
        }
        info->np = hi[0];
        info->nfixed = hi[1];
        info->nmoving = hi[2];
        info->nfloat = hi[3];
        info->nfluidout = hi[4];
        info->time = ts;
    }
    if (info->np < 0 || info->nfixed < 0 || info->nmoving < 0 || info->nfloat < 0 || info->nfluidout < 0 ||
        info->nfluidout > info->np || info->nfixed + info->nmoving + info->nfloat > info->np)
        return record_error(SPHMP_ERR_INVALID_ARG, "inconsistent .bi2 particle counts");
    info->nbound = info->nfixed + info->nmoving + info->nfloat;
    info->nfluid = info->np - info->nbound;
    if (!pos && !vel && !rhop) return SPHMP_OK;  // head only
    if (cap < info->np) return record_error(SPHMP_ERR_CAPACITY, "arrays smaller than the file's particle count");
    const int32_t npok = info->np - info->nfluidout;
    // particles the file does not carry (fixed ones of a short file, fluid that left) read as zero
    std::vector<float> p3((size_t)info->np * 3, 0.f), v3((size_t)info->np * 3, 0.f), r((size_t)info->np, 0.f);
    const int32_t first = info->full ? 0 : info->nfixed;
    const size_t nmov = (size_t)(npok - first);
    if (!read_exact(f.f, p3.data() + (size_t)first * 3, nmov * 12) ||
        !read_exact(f.f, v3.data() + (size_t)first * 3, nmov * 12) || !read_exact(f.f, r.data(), (size_t)npok * 4))
        return record_error(SPHMP_ERR_INVALID_ARG, "truncated .bi2 particle data");
    if (swap) {
        swap32(p3.data() + (size_t)first * 3, nmov * 3);
        swap32(v3.data() + (size_t)first * 3, nmov * 3);
        swap32(r.data(), (size_t)npok);
    }
    if (pos) memcpy(pos, p3.data(), p3.size() * 4);
    if (vel) memcpy(vel, v3.data(), v3.size() * 4);
    if (rhop) memcpy(rhop, r.data(), r.size() * 4);
    return SPHMP_OK;
}

sphmp_status sphmp_add_bi2_shape(const sphmp_params* p, const float* pos, int32_t np, float scale,
                                 const float offs[3], const float vel[3], int32_t phase, sphmp_display_pack* disp,
                                 sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    if (!p || (np > 0 && !pos) || !offs || !vel || !disp || !calc || !count || np < 0 || !(scale != 0.f) ||
        phase < 0 || phase >= SPHMP_MAX_PHASES)
        return record_error(SPHMP_ERR_INVALID_ARG, "bad arguments");
    if (*count < 0 || *count > cap || np > cap - *count)
        return record_error(SPHMP_ERR_CAPACITY, "shape does not fit the record arrays");
    // FluidSystem::AddShape (SPH_Solver/fluids/fluid_system.cpp:809-835): file (x, y, z)
    // divided by the scale becomes (x, z, y) plus the offset
    for (int32_t i = 0; i < np; i++) {
        const int32_t k = (*count)++;
        sphmp_display_pack& d = disp[k];
        sphmp_calc_pack& c = calc[k];
        memset(&d, 0, sizeof(d));
        memset(&c, 0, sizeof(c));
        c.deformGrad[0] = c.deformGrad[4] = c.deformGrad[8] = 1.0f;  // as AddParticle
        const float x = pos[3 * i] / scale, z = pos[3 * i + 1] / scale, y = pos[3 * i + 2] / scale;
        d.pos[0] = x + offs[0];
        d.pos[1] = y + offs[1];
        d.pos[2] = z + offs[2];
        d.color[0] = 0.2f;
        d.color[1] = 0.5f;
        d.color[2] = 0.8f;
        d.color[3] = 0.5f;
        d.type = SPHMP_TYPE_FLUID;
        for (int a = 0; a < 3; a++) c.vel[a] = vel[a];
        c.restdens = p->densArr[phase];
        c.mass = p->massArr[phase];
        c.visc = p->viscArr[phase];
        c.bornid = k;
    }
    return SPHMP_OK;
}

// State checkpoint, little endian:
//   "SPHMPST1", uint32 version (1), int32 n, int32 nphase, uint32 0,
//   n display records (32 B), n calculation records (224 B),
//   n x 3 float volume fractions, n x 3 float (g - a) of the last step.
sphmp_status sphmp_save_state(sphmp_ctx* ctx, const char* path) {
    if (!ctx || !path) return record_error(SPHMP_ERR_INVALID_ARG, "bad arguments");
    if (!host_little_endian()) return record_error(SPHMP_ERR_INVALID_ARG, "checkpoints are written on little-endian hosts");
    const int32_t n = sphmp_num_particles(ctx);
    sphmp_params prm;
    if (sphmp_status st = sphmp_get_params(ctx, &prm)) return st;
    std::vector<sphmp_display_pack> disp((size_t)n > 0 ? n : 1);
    std::vector<sphmp_calc_pack> calc((size_t)n > 0 ? n : 1);
    std::vector<float> alpha((size_t)n * 3 + 1), aprev((size_t)n * 3 + 1);
    if (n > 0) {
        if (sphmp_status st = sphmp_download_aos(ctx, disp.data(), calc.data(), n)) return st;
        if (sphmp_status st = sphmp_download_field(ctx, SPHMP_F_ALPHA, alpha.data(), n)) return st;
        if (sphmp_status st = sphmp_download_field(ctx, SPHMP_F_APREV, aprev.data(), n)) return st;
    }
    File f(fopen(path, "wb"));
    if (!f.f) return record_error(SPHMP_ERR_INVALID_ARG, "cannot open the checkpoint for writing");
    const uint32_t version = 1, zero = 0;
    const int32_t nphase = prm.nphase;
    bool ok = fwrite("SPHMPST1", 1, 8, f.f) == 8 && fwrite(&version, 4, 1, f.f) == 1 && fwrite(&n, 4, 1, f.f) == 1 &&
              fwrite(&nphase, 4, 1, f.f) == 1 && fwrite(&zero, 4, 1, f.f) == 1;
    if (ok && n > 0)
        ok = fwrite(disp.data(), sizeof(sphmp_display_pack), n, f.f) == (size_t)n &&
             fwrite(calc.data(), sizeof(sphmp_calc_pack), n, f.f) == (size_t)n &&
             fwrite(alpha.data(), 12, n, f.f) == (size_t)n && fwrite(aprev.data(), 12, n, f.f) == (size_t)n;
    if (!ok) return record_error(SPHMP_ERR_INVALID_ARG, "write error on the checkpoint");
    return SPHMP_OK;
}

sphmp_status sphmp_load_state(sphmp_ctx* ctx, const char* path) {
    if (!ctx || !path) return record_error(SPHMP_ERR_INVALID_ARG, "bad arguments");
    if (!host_little_endian()) return record_error(SPHMP_ERR_INVALID_ARG, "checkpoints are read on little-endian hosts");
    File f(fopen(path, "rb"));
    if (!f.f) return record_error(SPHMP_ERR_INVALID_ARG, "cannot open the checkpoint");
    char magic[8];
    uint32_t version = 0, zero = 0;
    int32_t n = 0, nphase = 0;
    if (!read_exact(f.f, magic, 8) || memcmp(magic, "SPHMPST1", 8) != 0 || !read_exact(f.f, &version, 4) ||
        version != 1 || !read_exact(f.f, &n, 4) || !read_exact(f.f, &nphase, 4) || !read_exact(f.f, &zero, 4))
        return record_error(SPHMP_ERR_INVALID_ARG, "not a version-1 sphmp checkpoint");
    sphmp_params prm;
    if (sphmp_status st = sphmp_get_params(ctx, &prm)) return st;
    if (nphase != prm.nphase) return record_error(SPHMP_ERR_INVALID_ARG, "checkpoint phase count differs from the context's");
    if (n < 0 || n > prm.maxNum) return record_error(SPHMP_ERR_CAPACITY, "checkpoint larger than the context's capacity");
    std::vector<sphmp_display_pack> disp((size_t)n > 0 ? n : 1);
    std::vector<sphmp_calc_pack> calc((size_t)n > 0 ? n : 1);
    std::vector<float> alpha((size_t)n * 3 + 1), aprev((size_t)n * 3 + 1);
    if (n > 0 && !(read_exact(f.f, disp.data(), sizeof(sphmp_display_pack) * (size_t)n) &&
                   read_exact(f.f, calc.data(), sizeof(sphmp_calc_pack) * (size_t)n) &&
                   read_exact(f.f, alpha.data(), 12 * (size_t)n) && read_exact(f.f, aprev.data(), 12 * (size_t)n)))
        return record_error(SPHMP_ERR_INVALID_ARG, "truncated checkpoint");
    if (sphmp_status st = sphmp_upload_aos(ctx, disp.data(), calc.data(), n)) return st;
    if (n > 0) {
        if (sphmp_status st = sphmp_upload_field(ctx, SPHMP_F_ALPHA, alpha.data(), n)) return st;
        if (sphmp_status st = sphmp_upload_field(ctx, SPHMP_F_APREV, aprev.data(), n)) return st;
    }
    return SPHMP_OK;
}

}  // extern "C"
