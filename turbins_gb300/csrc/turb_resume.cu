// turb_resume.cu -- host side of the restart files, in the reference's
// formats (Resume.c):
//  * 3-D fields: PETSc binary vectors as Resume_write_data writes them through
//    VecView (PETSc 3.1, VecView_Seq_Binary): the int32 pair
//    {VEC_FILE_COOKIE = 1211214, N} then N doubles, every word big-endian; on
//    one rank a DA vector's natural order is the DA order [k][j][i];
//  * Resume_primary.dat: the text of Resume_write_primary_data
//    (Resume.c:248-279), "time=\n%lf\ndt=\n%lf\ndt_old=\n%lf\niteration=\n%d\n
//    output_iter=\n%d\n";
//  * 2-D [NZ][NX] arrays: raw native doubles (Resume_write_2D_data,
//    Resume.c:321-351).
// Byte order is handled with shifts, so the code is the same on little- and
// big-endian hosts.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/turbins_gb300.h"

namespace {

constexpr int32_t VEC_COOKIE = 1211214;

void be32(unsigned char *b, uint32_t x)
{
    for (int i = 0; i < 4; i++) b[i] = (unsigned char)(x >> (24 - 8 * i));
}
uint32_t rd_be32(const unsigned char *b)
{
    return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}
void be64(unsigned char *b, double v)
{
    uint64_t x;
    memcpy(&x, &v, 8);
    for (int i = 0; i < 8; i++) b[i] = (unsigned char)(x >> (56 - 8 * i));
}
double rd_be64(const unsigned char *b)
{
    uint64_t x = 0;
    for (int i = 0; i < 8; i++) x = (x << 8) | b[i];
    double v;
    memcpy(&v, &x, 8);
    return v;
}

struct File {
    FILE *f;
    File(const char *p, const char *m) : f(fopen(p, m)) {}
    ~File() { if (f) fclose(f); }
};

}  // namespace

// header + payload already in file byte order (big-endian words)
int petsc_vec_write_be(const char *path, const void *be_words, long long n)
{
    File o(path, "wb");
    if (!o.f) return TURB_ERR_IO;
    unsigned char h[8];
    be32(h, (uint32_t)VEC_COOKIE);
    be32(h + 4, (uint32_t)n);
    if (fwrite(h, 1, 8, o.f) != 8) return TURB_ERR_IO;
    if (fwrite(be_words, 8, (size_t)n, o.f) != (size_t)n) return TURB_ERR_IO;
    return TURB_OK;
}

// checks the header, leaves the payload in file byte order
int petsc_vec_read_be(const char *path, void *be_words, long long n)
{
    File in(path, "rb");
    if (!in.f) return TURB_ERR_IO;
    unsigned char h[8];
    if (fread(h, 1, 8, in.f) != 8) return TURB_ERR_IO;
    if ((int32_t)rd_be32(h) != VEC_COOKIE || (long long)rd_be32(h + 4) != n) return TURB_ERR_FORMAT;
    if (fread(be_words, 8, (size_t)n, in.f) != (size_t)n) return TURB_ERR_IO;
    return TURB_OK;
}

std::string resume_path(const char *dir, const char *name)
{
    std::string p = dir && *dir ? dir : ".";
    if (p.back() != '/') p += '/';
    return p + name;
}

extern "C" {

int turb_petsc_vec_write(const char *path, const double *data, long long n)
{
    if (!path || (!data && n) || n < 0 || n > 0x7fffffffLL) return TURB_ERR_ARG;
    std::vector<unsigned char> buf((size_t)n * 8);
    for (long long t = 0; t < n; t++) be64(&buf[(size_t)t * 8], data[t]);
    return petsc_vec_write_be(path, buf.data(), n);
}

int turb_petsc_vec_read(const char *path, double *data, long long n)
{
    if (!path || (!data && n) || n < 0 || n > 0x7fffffffLL) return TURB_ERR_ARG;
    std::vector<unsigned char> buf((size_t)n * 8);
    int rc = petsc_vec_read_be(path, buf.data(), n);
    if (rc) return rc;
    for (long long t = 0; t < n; t++) data[t] = rd_be64(&buf[(size_t)t * 8]);
    return TURB_OK;
}

int turb_resume_primary_write(const char *dir, const turb_primary *p)
{
    if (!p) return TURB_ERR_ARG;
    File o(resume_path(dir, "Resume_primary.dat").c_str(), "w");
    if (!o.f) return TURB_ERR_IO;
    if (fprintf(o.f, "time=\n%lf\ndt=\n%lf\ndt_old=\n%lf\niteration=\n%d\noutput_iter=\n%d\n", p->time, p->dt,
                p->dt_old, p->iter, p->output_iter) < 0)
        return TURB_ERR_IO;
    return TURB_OK;
}

int turb_resume_primary_read(const char *dir, turb_primary *p)
{
    if (!p) return TURB_ERR_ARG;
    File in(resume_path(dir, "Resume_primary.dat").c_str(), "r");
    if (!in.f) return TURB_ERR_IO;
    char s[5][64];
    turb_primary q;
    int n = fscanf(in.f, "%63s\n%lf\n%63s\n%lf\n%63s\n%lf\n%63s\n%d\n%63s\n%d", s[0], &q.time, s[1], &q.dt, s[2],
                   &q.dt_old, s[3], &q.iter, s[4], &q.output_iter);
    if (n != 10) return TURB_ERR_FORMAT;
    *p = q;
    return TURB_OK;
}

int turb_resume_2d_write(const char *path, const double *data, int nx, int nz)
{
    if (!path || !data || nx <= 0 || nz <= 0) return TURB_ERR_ARG;
    File o(path, "wb");
    if (!o.f) return TURB_ERR_IO;
    size_t n = (size_t)nx * nz;
    return fwrite(data, sizeof(double), n, o.f) == n ? TURB_OK : TURB_ERR_IO;
}

int turb_resume_2d_read(const char *path, double *data, int nx, int nz)
{
    if (!path || !data || nx <= 0 || nz <= 0) return TURB_ERR_ARG;
    File in(path, "rb");
    if (!in.f) return TURB_ERR_IO;
    size_t n = (size_t)nx * nz;
    return fread(data, sizeof(double), n, in.f) == n ? TURB_OK : TURB_ERR_IO;
}

}  // extern "C"
