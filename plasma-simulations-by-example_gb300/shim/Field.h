/*
 * Field.h (drop-in) -- vec3 and the node-centred Field_ container with the
 * interface of the reference's Field.h (ch2/Field.h:7-231,
 * ch3/ver2/Field.h:55-247), backed by libespic.
 *
 * Storage is one contiguous host array in the reference's U order
 * (u = k*ni*nj + j*ni + i, ch3/ver2/Field.h:161).  A Field_ owned by a World
 * or Species is a mirror of a device field: reads pull the device copy when
 * it is newer, and any non-const access marks the mirror dirty so that it is
 * pushed before the next device operation.  f[i][j][k] works through small
 * proxy objects (the reference returns T**).
 */
#ifndef ESPIC_SHIM_FIELD_H
#define ESPIC_SHIM_FIELD_H

#include <cmath>
#include <cstdint>
#include <functional>
#include <memory>
#include <ostream>
#include <utility>
#include <vector>

template <typename T>
struct vec3 {
    vec3(const T u, const T v, const T w) : d{u, v, w} {}
    vec3(const T a[3]) : d{a[0], a[1], a[2]} {}
    vec3() : d{0, 0, 0} {}
    T &operator[](int i) { return d[i]; }
    T operator()(int i) const { return d[i]; }
    vec3<T> &operator=(double s) {
        d[0] = s;
        d[1] = s;
        d[2] = s;
        return *this;
    }
    vec3<T> &operator+=(vec3<T> o) {
        d[0] += o[0];
        d[1] += o[1];
        d[2] += o[2];
        return *this;
    }
    vec3<T> &operator-=(vec3<T> o) {
        d[0] -= o[0];
        d[1] -= o[1];
        d[2] -= o[2];
        return *this;
    }
    /* ch4/Field.h:17-34: division by a scalar, dot, mag, unit, cross */
    vec3<T> operator/(double s) const { return vec3<T>(d[0] / s, d[1] / s, d[2] / s); }
    vec3<T> &operator/=(double s) {
        d[0] /= s;
        d[1] /= s;
        d[2] /= s;
        return *this;
    }
    friend T dot(const vec3<T> &v1, const vec3<T> &v2) {
        T s = 0;
        for (int i = 0; i < 3; i++) s += v1(i) * v2(i);
        return s;
    }
    friend T mag(const vec3<T> &v) { return std::sqrt(dot(v, v)); }
    friend vec3<T> unit(const vec3<T> &v) { return vec3<T>(v) / mag(v); }
    friend vec3<T> cross(const vec3<T> &a, const vec3<T> &b) {
        return vec3<T>(a(1) * b(2) - a(2) * b(1), a(2) * b(0) - a(0) * b(2), a(0) * b(1) - a(1) * b(0));
    }

protected:
    T d[3];
};

template <typename T>
vec3<T> operator+(const vec3<T> &a, const vec3<T> &b) {
    return vec3<T>(a(0) + b(0), a(1) + b(1), a(2) + b(2));
}
template <typename T>
vec3<T> operator-(const vec3<T> &a, const vec3<T> &b) {
    return vec3<T>(a(0) - b(0), a(1) - b(1), a(2) - b(2));
}
template <typename T>
vec3<T> operator*(const vec3<T> &a, const vec3<T> &b) {
    return vec3<T>(a(0) * b(0), a(1) * b(1), a(2) * b(2));
}
template <typename T>
vec3<T> operator/(const vec3<T> &a, const vec3<T> &b) {
    return vec3<T>(a(0) / b(0), a(1) / b(1), a(2) / b(2));
}
template <typename T>
vec3<T> operator*(const vec3<T> &a, T s) {
    return vec3<T>(a(0) * s, a(1) * s, a(2) * s);
}
template <typename T>
vec3<T> operator*(T s, const vec3<T> &a) {
    return vec3<T>(a(0) * s, a(1) * s, a(2) * s);
}
template <typename T>
std::ostream &operator<<(std::ostream &out, vec3<T> &v) {
    out << v[0] << " " << v[1] << " " << v[2];
    return out;
}

using double3 = vec3<double>;
using int3 = vec3<int>;

/* The link between a host mirror and its device field. */
struct FieldLink {
    std::function<void(void *)> pull;       /* device -> host (whole field) */
    std::function<void(const void *)> push; /* host -> device (whole field) */
    uint64_t device_version = 1;            /* bumped by device writers */
    uint64_t host_version = 0;              /* device_version the host holds */
    bool host_dirty = false;                /* host edits not yet pushed */
};

template <typename T>
class Field_ {
public:
    Field_(int ni, int nj, int nk) : ni{ni}, nj{nj}, nk{nk}, data((size_t)ni * nj * nk) { clear(); }
    Field_(int3 nn) : Field_(nn(0), nn(1), nn(2)) {}
    Field_(const Field_ &other) : ni{other.ni}, nj{other.nj}, nk{other.nk} {
        other.pull();
        data = other.data;
    }
    Field_(Field_ &&other) : ni{other.ni}, nj{other.nj}, nk{other.nk}, data(std::move(other.data)),
                             link(std::move(other.link)) {}
    /* the reference's move assignment does nothing (ch2/Field.h:92) */
    Field_ &operator=(Field_ &&) { return *this; }

    struct Row {
        Field_ *f;
        int i, j;
        T &operator[](int k) { return f->data[f->U(i, j, k)]; }
    };
    struct Plane {
        Field_ *f;
        int i;
        Row operator[](int j) { return Row{f, i, j}; }
    };
    /* f[i][j][k]: pulls, then counts as a write */
    Plane operator[](int i) {
        pull();
        mark_dirty();
        return Plane{this, i};
    }
    T operator()(int i, int j, int k) const {
        pull();
        return data[U(i, j, k)];
    }

    void operator=(double s) {
        for (auto &x : data) x = s;
        if (link) {
            link->host_version = link->device_version;
            link->host_dirty = true;
        }
    }
    void operator/=(const Field_ &other) {
        pull();
        other.pull();
        for (size_t u = 0; u < data.size(); u++) {
            if (other.data[u] != 0)
                data[u] /= other.data[u];
            else
                data[u] = 0;
        }
        mark_dirty();
    }
    Field_ &operator+=(const Field_ &other) {
        pull();
        other.pull();
        for (size_t u = 0; u < data.size(); u++) data[u] += other.data[u];
        mark_dirty();
        return *this;
    }
    Field_ &operator*=(double s) {
        pull();
        for (auto &x : data) x *= s;
        mark_dirty();
        return *this;
    }
    friend Field_<T> operator*(double s, const Field_<T> &f) {
        Field_<T> r(f);
        return r *= s;
    }

    int U(int i, int j, int k) const { return k * ni * nj + j * ni + i; }
    void clear() { (*this) = 0; }

    /* Field_::scatter / gather (ch3/ver2/Field.h:167-209), on the host mirror */
    void scatter(double3 lc, T value) {
        int i = (int)lc[0], j = (int)lc[1], k = (int)lc[2];
        double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
        Plane p = (*this)[i];
        Plane q = Plane{this, i + 1};
        p[j][k] += (T)value * (1 - di) * (1 - dj) * (1 - dk);
        q[j][k] += (T)value * (di) * (1 - dj) * (1 - dk);
        q[j + 1][k] += (T)value * (di) * (dj) * (1 - dk);
        p[j + 1][k] += (T)value * (1 - di) * (dj) * (1 - dk);
        p[j][k + 1] += (T)value * (1 - di) * (1 - dj) * (dk);
        q[j][k + 1] += (T)value * (di) * (1 - dj) * (dk);
        q[j + 1][k + 1] += (T)value * (di) * (dj) * (dk);
        p[j + 1][k + 1] += (T)value * (1 - di) * (dj) * (dk);
    }
    T gather(double3 lc) {
        pull();
        int i = (int)lc[0], j = (int)lc[1], k = (int)lc[2];
        double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
        return data[U(i, j, k)] * (1 - di) * (1 - dj) * (1 - dk) + data[U(i + 1, j, k)] * (di) * (1 - dj) * (1 - dk) +
               data[U(i + 1, j + 1, k)] * (di) * (dj) * (1 - dk) + data[U(i, j + 1, k)] * (1 - di) * (dj) * (1 - dk) +
               data[U(i, j, k + 1)] * (1 - di) * (1 - dj) * (dk) + data[U(i + 1, j, k + 1)] * (di) * (1 - dj) * (dk) +
               data[U(i + 1, j + 1, k + 1)] * (di) * (dj) * (dk) + data[U(i, j + 1, k + 1)] * (1 - di) * (dj) * (dk);
    }
    /* Field_::updateAverage (ch3/ver2/Field.h:214-220), on the host */
    void updateAverage(const Field_ &I) {
        pull();
        I.pull();
        for (size_t u = 0; u < data.size(); u++)
            data[u] = (I.data[u] + ave_samples * data[u]) / (ave_samples + 1);
        ++ave_samples;
        mark_dirty();
    }

    template <typename S>
    friend std::ostream &operator<<(std::ostream &out, Field_<S> &f);

    const int ni, nj, nk;

    /* ---- mirror plumbing (used by the drop-in World and Species) ---- */
    void bind(std::function<void(void *)> pull_fn, std::function<void(const void *)> push_fn) {
        link.reset(new FieldLink());
        link->pull = std::move(pull_fn);
        link->push = std::move(push_fn);
    }
    /* the device copy changed */
    void device_written() {
        if (!link) return;
        if (link->host_dirty) push();
        link->device_version++;
    }
    /* push host edits before a device operation reads the field */
    void push() {
        if (link && link->host_dirty) {
            link->push(data.data());
            link->host_dirty = false;
        }
    }
    void pull() const {
        if (link && !link->host_dirty && link->host_version != link->device_version) {
            link->pull(data.data());
            link->host_version = link->device_version;
        }
    }
    const T *host_data() const {
        pull();
        return data.data();
    }

protected:
    void mark_dirty() {
        if (link) link->host_dirty = true;
    }
    mutable std::vector<T> data;
    std::unique_ptr<FieldLink> link;
    int ave_samples = 0;
};

/* writes out data k outer, j, i inner (ch2/Field.h:218-225) */
template <typename T>
std::ostream &operator<<(std::ostream &out, Field_<T> &f) {
    f.pull();
    for (int k = 0; k < f.nk; k++, out << "\n")
        for (int j = 0; j < f.nj; j++)
            for (int i = 0; i < f.ni; i++) out << f.data[f.U(i, j, k)] << " ";
    return out;
}

using Field = Field_<double>;
using FieldI = Field_<int>;
using Field3 = Field_<double3>;
using dvector = std::vector<double>;

#endif
