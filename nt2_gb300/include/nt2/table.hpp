// nt2/table.hpp -- NT2's table/expression surface over the GB300 evaluator.
//
// A Boost-free C++17 restatement of the part of NT2's container DSL the
// fused-expression hot path uses, evaluated by libnt2gpu through its C ABI
// (include/nt2g.h):
//
//   nt2::table<float, nt2::device_> S(nt2::of_size(n)), K(...), T(...), C, P;
//   nt2::tie(C, P) = nt2::tie(nt2::fnms(e, nt2::normcdf(d2), S*nt2::normcdf(d1)), ...);
//   float s = nt2::globalsum(X*Y);
//
// What it mirrors (paths inside the NT2 tree):
//   table<T,S>            modules/core/container/table/include/nt2/core/container/table/table.hpp:34-171
//   locality host/device  modules/core/sdk/include/nt2/core/settings/locality.hpp:16-63
//   run_assign->transform modules/core/base/include/nt2/dsl/functions/elementwise/run.hpp:21-36
//   tie                   modules/core/container/table/include/nt2/core/functions/expr/tie.hpp:40-182
//   transform(out,in,rng) modules/core/container/table/include/nt2/core/functions/expr/transform.hpp:22-60
//   sum / dot / globalsum modules/core/reduction/include/nt2/reduction/functions/expr/dot.hpp:22-42,
//                         modules/core/reduction/include/nt2/core/functions/globalsum.hpp:43-45
//
// NT2 captures an expression as a Boost.Proto tree at compile time and lets
// the outermost site (cuda_<...> when NT2_HAS_CUDA) pick the evaluator.  Here
// the tree is captured at run time, lowered to an SSA program, compiled once
// per distinct program by the library (which binds the named expressions to
// their fused kernels) and evaluated in one pass on the device.  Host tables
// in an expression are staged to the device and back, the role of NT2's
// host/device assignment copies (modules/arch/cuda/include/nt2/memory/
// functions/cuda/copy.hpp:52-86).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "nt2g.h"

namespace nt2 {

// ------------------------------------------------------------------ errors --
struct gpu_error : std::runtime_error {
    nt2g_status status;
    gpu_error(nt2g_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

inline void check(nt2g_status s, const char *what)
{
    if (s != NT2G_OK) throw gpu_error(s, std::string(what) + ": " + nt2g_last_error());
}

// ---------------------------------------------------------------- settings --
struct host_ {};
struct device_ {};

struct of_size_ {
    std::size_t d[4] = {1, 1, 1, 1};
    std::size_t numel() const { return d[0] * d[1] * d[2] * d[3]; }
};
inline of_size_ of_size(std::size_t a, std::size_t b = 1, std::size_t c = 1, std::size_t e = 1)
{
    of_size_ s;
    s.d[0] = a; s.d[1] = b; s.d[2] = c; s.d[3] = e;
    return s;
}

// Evaluation options: arithmetic policy and the stream every call uses, per
// host thread (each thread evaluates on its own stream; a new thread starts
// with the fast policy on the default stream).
struct gpu_options {
    int precision = NT2G_PREC_FAST;
    void *stream = nullptr;
};
inline gpu_options &options()
{
    thread_local gpu_options o;
    return o;
}

namespace detail {

template <class T> struct dtype_of;
template <> struct dtype_of<float> { static constexpr int value = NT2G_F32; };
template <> struct dtype_of<std::uint8_t> { static constexpr int value = NT2G_U8; };

// One expression node.  Leaves hold a table (by storage pointer) or a scalar.
struct node {
    int op = 0;       // nt2g_opcode
    int dtype = NT2G_F32;
    float imm = 0.f;  // CONST value
    const void *table_key = nullptr;   // identity of a table leaf
    void *dev_ptr = nullptr;           // device storage of a device table leaf
    const void *host_ptr = nullptr;    // host storage of a host table leaf
    std::size_t numel = 0;
    std::size_t ext[4] = {0, 0, 0, 0};  // extent of a table leaf
    std::shared_ptr<node> a, b, c;
};
using node_ptr = std::shared_ptr<node>;

inline node_ptr make(int op, int dt, node_ptr a = {}, node_ptr b = {}, node_ptr c = {})
{
    auto n = std::make_shared<node>();
    n->op = op; n->dtype = dt; n->a = std::move(a); n->b = std::move(b); n->c = std::move(c);
    return n;
}

// device buffer with RAII
struct device_buffer {
    void *p = nullptr;
    std::size_t bytes = 0;
    device_buffer() = default;
    explicit device_buffer(std::size_t n) : bytes(n) { check(nt2g_device_alloc(n, &p), "device allocation"); }
    ~device_buffer() { if (p) nt2g_device_free(p); }
    device_buffer(const device_buffer &) = delete;
    device_buffer &operator=(const device_buffer &) = delete;
    device_buffer(device_buffer &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    device_buffer &operator=(device_buffer &&o) noexcept
    {
        if (this != &o) { if (p) nt2g_device_free(p); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
};

}  // namespace detail

// An expression of element type T (float or uint8 arithmetic; comparisons
// give a logical expression that conditions consume).
template <class T> struct expr {
    detail::node_ptr n;
    bool logical = false;
};

template <class T, class Site = host_> class table;

namespace detail {

template <class T, class S> node_ptr leaf(const table<T, S> &t);

template <class T> node_ptr lift(const expr<T> &e) { return e.n; }
template <class T, class S> node_ptr lift(const table<T, S> &t) { return leaf(t); }
template <class T> node_ptr lift_scalar(T v)
{
    auto n = make(NT2G_OP_CONST, dtype_of<T>::value);
    n->imm = (float)v;
    return n;
}

template <class X> struct elem_of;
template <class T> struct elem_of<expr<T>> { using type = T; };
template <class T, class S> struct elem_of<table<T, S>> { using type = T; };

template <class X, class = void> struct is_nt2 : std::false_type {};
template <class X> struct is_nt2<X, std::void_t<typename elem_of<std::decay_t<X>>::type>> : std::true_type {};

// element type of the first nt2 operand; no `type` (so overloads drop out)
// when no operand is a table or an expression
template <class A, class B, class = void> struct common {};
template <class A, class B> struct common<A, B, std::enable_if_t<is_nt2<A>::value>> {
    using type = typename elem_of<std::decay_t<A>>::type;
};
template <class A, class B> struct common<A, B, std::enable_if_t<!is_nt2<A>::value && is_nt2<B>::value>> {
    using type = typename elem_of<std::decay_t<B>>::type;
};
template <class A, class B, class C, class = void> struct common3 : common<B, C> {};
template <class A, class B, class C> struct common3<A, B, C, std::enable_if_t<is_nt2<A>::value>> {
    using type = typename elem_of<std::decay_t<A>>::type;
};

template <class T, class X> node_ptr any(const X &x)
{
    if constexpr (is_nt2<X>::value) return lift(x);
    else return lift_scalar<T>((T)x);
}

}  // namespace detail

// ------------------------------------------------------------------- table --
template <class T, class Site> class table {
    static_assert(std::is_same<T, float>::value || std::is_same<T, std::uint8_t>::value,
                  "tables of float or uint8 are evaluated on the GPU");

public:
    using value_type = T;
    static constexpr bool on_device = std::is_same<Site, device_>::value;

    table() = default;
    explicit table(of_size_ s) { resize(s); }
    table(const table &o) { *this = o; }
    table(table &&) noexcept = default;
    table &operator=(table &&) noexcept = default;

    table &operator=(const table &o)
    {
        if (this == &o) return *this;
        resize(o.size_);
        copy_from(o);
        return *this;
    }

    template <class S2> table &operator=(const table<T, S2> &o)
    {
        resize(o.extent());
        copy_from(o);
        return *this;
    }

    // R = expression  (run_assign -> transform over the whole table)
    table &operator=(const expr<T> &e);

    void resize(of_size_ s)
    {
        if (s.numel() == numel()) { size_ = s; return; }
        size_ = s;
        if constexpr (on_device) dev_ = detail::device_buffer(s.numel() * sizeof(T));
        else host_.assign(s.numel(), T());
    }

    of_size_ extent() const { return size_; }
    std::size_t numel() const { return size_.numel(); }
    std::size_t size(int dim) const { return size_.d[dim - 1]; }

    T *data() { return on_device ? (T *)dev_.p : host_.data(); }
    const T *data() const { return on_device ? (const T *)dev_.p : host_.data(); }

    // 1-based element access on host tables (NT2 indexing)
    T &operator()(std::size_t i)
    {
        static_assert(!on_device, "element access on a device table: copy it to a host table first");
        return host_[i - 1];
    }
    const T &operator()(std::size_t i) const
    {
        static_assert(!on_device, "element access on a device table: copy it to a host table first");
        return host_[i - 1];
    }
    T &operator()(std::size_t i, std::size_t j) { return (*this)(i + (j - 1) * size_.d[0]); }

private:
    template <class U, class S2> friend class table;

    template <class S2> void copy_from(const table<T, S2> &o)
    {
        const std::size_t bytes = numel() * sizeof(T);
        if (!bytes) return;
        constexpr bool src_dev = table<T, S2>::on_device;
        if constexpr (on_device && src_dev)
            check(nt2g_memcpy(data(), o.data(), bytes, 3, options().stream), "device copy");
        else if constexpr (on_device)
            check(nt2g_memcpy(data(), o.data(), bytes, 1, options().stream), "host->device copy");
        else if constexpr (src_dev) {
            check(nt2g_memcpy(data(), o.data(), bytes, 2, options().stream), "device->host copy");
            check(nt2g_stream_synchronize(options().stream), "device->host copy");
        } else
            std::memcpy(data(), o.data(), bytes);
    }

    of_size_ size_ = of_size(0);
    std::vector<T> host_;
    detail::device_buffer dev_;
};

namespace detail {

template <class T, class S> node_ptr leaf(const table<T, S> &t)
{
    auto n = make(NT2G_OP_LOAD, dtype_of<T>::value);
    n->table_key = t.data();
    n->numel = t.numel();
    for (int k = 0; k < 4; ++k) n->ext[k] = t.extent().d[k];
    if constexpr (table<T, S>::on_device) n->dev_ptr = (void *)t.data();
    else n->host_ptr = t.data();
    return n;
}

// ------------------------------------------------------------ lowering ----
struct lowered {
    std::vector<nt2g_op> ops;
    std::vector<const node *> slot_leaf;  // slot -> leaf node (tables)
    std::string key;
};

struct lowering {
    lowered L;
    std::map<const void *, int> slot_of;   // table identity -> slot
    std::map<const node *, int> value_of;  // non-leaf node -> SSA value

    int slot(const node *leafn)
    {
        auto it = slot_of.find(leafn->table_key);
        if (it != slot_of.end()) return it->second;
        int s = (int)L.slot_leaf.size();
        slot_of[leafn->table_key] = s;
        L.slot_leaf.push_back(leafn);
        return s;
    }

    int push(int code, int dt, int a = -1, int b = -1, int c = -1, float imm = 0.f)
    {
        nt2g_op o;
        o.code = (int16_t)code; o.dtype = (int16_t)dt; o.a = a; o.b = b; o.c = c; o.imm = imm;
        L.ops.push_back(o);
        return (int)L.ops.size() - 1;
    }

    int emit(const node *n)
    {
        if (n->op == NT2G_OP_LOAD)  // loads are not memoised: tie() may store the table first
            return push(NT2G_OP_LOAD, n->dtype, slot(n));
        auto it = value_of.find(n);
        if (it != value_of.end()) return it->second;
        int v;
        if (n->op == NT2G_OP_CONST) v = push(NT2G_OP_CONST, n->dtype, -1, -1, -1, n->imm);
        else {
            int a = n->a ? emit(n->a.get()) : -1;
            int b = n->b ? emit(n->b.get()) : -1;
            int c = n->c ? emit(n->c.get()) : -1;
            v = push(n->op, n->dtype, a, b, c);
        }
        value_of[n] = v;
        return v;
    }

    void store(int v, const node *out_leaf, int dt)
    {
        push(NT2G_OP_STORE, dt, v, slot(out_leaf));
    }

    void finish()
    {
        L.key.assign((const char *)L.ops.data(), L.ops.size() * sizeof(nt2g_op));
        L.key += std::to_string(L.slot_leaf.size());
    }
};

// Compiled programs, one per distinct lowered program text.
inline nt2g_program *program_for(const lowered &L)
{
    static std::mutex mu;
    static std::map<std::string, std::unique_ptr<nt2g_program, void (*)(nt2g_program *)>> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(L.key);
    if (it != cache.end()) return it->second.get();
    nt2g_program *p = nullptr;
    check(nt2g_program_create(L.ops.data(), (int32_t)L.ops.size(), (int32_t)L.slot_leaf.size(), &p),
          "program compile");
    cache.emplace(L.key, std::unique_ptr<nt2g_program, void (*)(nt2g_program *)>(p, nt2g_program_destroy));
    return p;
}

// The fused kernel (or "generic") a lowered assignment binds to, without
// evaluating it: a host-only call (the program compiler touches no GPU).
inline std::string bound_kernel(const std::vector<node_ptr> &outs, const std::vector<node_ptr> &exprs,
                                const std::vector<int> &out_dtypes)
{
    lowering lw;
    for (std::size_t k = 0; k < outs.size(); ++k) lw.store(lw.emit(exprs[k].get()), outs[k].get(), out_dtypes[k]);
    lw.finish();
    nt2g_program_info info;
    check(nt2g_program_info_get(program_for(lw.L), &info), "program info");
    return info.kernel_name;
}

// Whether host tables are evaluated in place (the device reads and writes
// pageable host memory directly), asked once per process.
inline bool host_in_place()
{
    static const bool v = [] {
        int32_t p = 0;
        return nt2g_host_access(&p) == NT2G_OK && p != 0;
    }();
    return v;
}

template <class V> inline bool has_host_leaf(const V &slots)
{
    for (const node *l : slots)
        if (!l->dev_ptr) return true;
    return false;
}

// Evaluate tie(outs) = tie(exprs) over [offset, offset + count).
inline void evaluate(const std::vector<node_ptr> &outs, const std::vector<node_ptr> &exprs,
                     const std::vector<int> &out_dtypes, std::size_t offset, std::size_t count)
{
    lowering lw;
    for (std::size_t k = 0; k < outs.size(); ++k) lw.store(lw.emit(exprs[k].get()), outs[k].get(), out_dtypes[k]);
    lw.finish();
    nt2g_program *prog = program_for(lw.L);
    // arguments: device tables directly; host tables in place when the device
    // reaches host memory (pageable memory access), else staged through
    // device buffers (inputs up, outputs down)
    const bool in_place = host_in_place();
    const auto &slots = lw.L.slot_leaf;
    std::vector<nt2g_arg> args(slots.size());
    std::vector<device_buffer> staging;
    staging.reserve(slots.size());
    std::vector<char> is_out(slots.size(), 0);
    for (const auto &o : outs) is_out[lw.slot_of[o->table_key]] = 1;
    void *st = options().stream;
    for (std::size_t s = 0; s < slots.size(); ++s) {
        const node *l = slots[s];
        nt2g_arg &a = args[s];
        a.dtype = l->dtype;
        a.kind = 0;
        a.scalar = 0.0;
        if (l->dev_ptr) {
            a.ptr = l->dev_ptr;
        } else if (in_place) {
            a.ptr = (void *)l->host_ptr;
        } else {
            const std::size_t esz = l->dtype == NT2G_U8 ? 1 : 4;
            staging.emplace_back(l->numel * esz);
            a.ptr = staging.back().p;
            check(nt2g_memcpy(a.ptr, l->host_ptr, l->numel * esz, 1, st), "stage host table");
        }
    }
    check(nt2g_eval(prog, args.data(), (int32_t)args.size(), (int64_t)offset, (int64_t)count, options().precision,
                    0, st),
          "evaluate");
    bool staged_out = false;
    for (std::size_t s = 0; s < slots.size(); ++s) {
        const node *l = slots[s];
        if (!l->dev_ptr && is_out[s] && !in_place) {
            const std::size_t esz = l->dtype == NT2G_U8 ? 1 : 4;
            check(nt2g_memcpy((void *)l->host_ptr, args[s].ptr, l->numel * esz, 2, st), "unstage host table");
            staged_out = true;
        }
    }
    // host tables are the caller's to read as soon as the assignment returns
    if (staged_out || !staging.empty() || (in_place && has_host_leaf(slots)))
        check(nt2g_stream_synchronize(st), "synchronize");
}

}  // namespace detail

namespace detail {
// Extent of an expression: the element count of its table leaves, which must
// agree (NT2 asserts the same in run_assign).
inline std::size_t extent_of(const node *n)
{
    if (n->op == NT2G_OP_LOAD || n->op == NT2G_OP_INDEX) return n->numel;
    if (n->op == NT2G_OP_CONST) return n->numel;  // ones / zeros carry a size; plain scalars 0
    std::size_t e = 0;
    for (const node *c : {n->a.get(), n->b.get(), n->c.get()}) {
        if (!c) continue;
        std::size_t ce = extent_of(c);
        if (ce && e && ce != e) throw gpu_error(NT2G_ERR_INVALID, "expression operands of different sizes");
        if (ce) e = ce;
    }
    return e;
}
}  // namespace detail

// R = expr: like NT2's run_assign (modules/core/base/include/nt2/dsl/functions/
// elementwise/run.hpp:21-36), resize R to the expression's extent, then
// transform over it.
template <class T, class Site> table<T, Site> &table<T, Site>::operator=(const expr<T> &e)
{
    const std::size_t n = detail::extent_of(e.n.get());
    if (n && n != numel()) resize(of_size(n));
    evaluate_into(*this, e);
    return *this;
}

// transform(out, expr [, {offset, count}]) with NT2's 0-based (offset, count) range
template <class T, class S>
void evaluate_into(table<T, S> &out, const expr<T> &e, std::pair<std::size_t, std::size_t> range = {0, (std::size_t)-1})
{
    std::size_t count = range.second == (std::size_t)-1 ? out.numel() - range.first : range.second;
    detail::evaluate({detail::leaf(out)}, {e.n}, {detail::dtype_of<T>::value}, range.first, count);
}

template <class T, class S, class X>
void transform(table<T, S> &out, const X &e, std::pair<std::size_t, std::size_t> range)
{
    evaluate_into(out, expr<T>{detail::lift(e)}, range);
}

// ------------------------------------------------------------------- tie ----
template <class... Tabs> struct tie_lhs {
    std::tuple<Tabs &...> outs;

    template <class... Es> tie_lhs &operator=(const std::tuple<Es...> &rhs)
    {
        static_assert(sizeof...(Es) == sizeof...(Tabs), "tie: as many expressions as tables");
        std::vector<detail::node_ptr> o, e;
        std::vector<int> dts;
        std::size_t n = 0;
        collect(o, dts, n, std::index_sequence_for<Tabs...>{});
        collect_rhs(rhs, e, std::index_sequence_for<Es...>{});
        detail::evaluate(o, e, dts, 0, n);
        return *this;
    }

    // outputs that are still empty take the extent of their expression
    template <class... Es> tie_lhs &operator=(std::tuple<Es...> &&rhs)
    {
        resize_outputs(rhs, std::index_sequence_for<Es...>{});
        return *this = static_cast<const std::tuple<Es...> &>(rhs);
    }

    // which kernel `tie(outs) = rhs` would run (host-only)
    template <class... Es> std::string explain(const std::tuple<Es...> &rhs)
    {
        std::vector<detail::node_ptr> o, e;
        std::vector<int> dts;
        std::size_t n = 0;
        collect(o, dts, n, std::index_sequence_for<Tabs...>{});
        collect_rhs(rhs, e, std::index_sequence_for<Es...>{});
        return detail::bound_kernel(o, e, dts);
    }

private:
    template <class Tup, std::size_t... I> void resize_outputs(const Tup &rhs, std::index_sequence<I...>)
    {
        ((std::get<I>(outs).numel() == 0
              ? std::get<I>(outs).resize(of_size(detail::extent_of(detail::lift(std::get<I>(rhs)).get())))
              : void()),
         ...);
    }

    template <std::size_t... I>
    void collect(std::vector<detail::node_ptr> &o, std::vector<int> &dts, std::size_t &n, std::index_sequence<I...>)
    {
        ((o.push_back(detail::leaf(std::get<I>(outs))),
          dts.push_back(detail::dtype_of<typename std::decay_t<decltype(std::get<I>(outs))>::value_type>::value),
          n = std::get<I>(outs).numel()),
         ...);
    }
    template <class Tup, std::size_t... I>
    static void collect_rhs(const Tup &rhs, std::vector<detail::node_ptr> &e, std::index_sequence<I...>)
    {
        (e.push_back(detail::lift(std::get<I>(rhs))), ...);
    }
};

template <class... Tabs> struct is_all_tables : std::conjunction<std::is_lvalue_reference<Tabs>...> {};

template <class... Xs> auto tie(Xs &&...xs)
{
    if constexpr ((... && (std::is_lvalue_reference<Xs &&>::value && !std::is_const<std::remove_reference_t<Xs>>::value &&
                           detail::is_nt2<Xs>::value && !std::is_same<std::decay_t<Xs>,
                           expr<typename detail::elem_of<std::decay_t<Xs>>::type>>::value)))
        return tie_lhs<std::remove_reference_t<Xs>...>{std::tie(xs...)};
    else
        return std::make_tuple(expr<typename detail::elem_of<std::decay_t<Xs>>::type>{detail::lift(xs)}...);
}

// -------------------------------------------------------------- operators --
#define NT2G_BINARY(OPNAME, CODE, LOGICAL)                                                                       \
    template <class A, class B, class T = typename detail::common<A, B>::type>                                  \
    expr<T> OPNAME(const A &a, const B &b)                                                                       \
    {                                                                                                            \
        return expr<T>{detail::make(CODE, detail::dtype_of<T>::value, detail::any<T>(a), detail::any<T>(b)),   \
                       LOGICAL};                                                                                 \
    }

NT2G_BINARY(operator+, NT2G_OP_ADD, false)
NT2G_BINARY(operator-, NT2G_OP_SUB, false)
NT2G_BINARY(operator*, NT2G_OP_MUL, false)
NT2G_BINARY(operator/, NT2G_OP_DIV, false)
NT2G_BINARY(operator<, NT2G_OP_LT, true)
NT2G_BINARY(operator>, NT2G_OP_GT, true)
NT2G_BINARY(operator<=, NT2G_OP_LE, true)
NT2G_BINARY(operator>=, NT2G_OP_GE, true)
NT2G_BINARY(operator==, NT2G_OP_EQ, true)
NT2G_BINARY(operator!=, NT2G_OP_NE, true)
NT2G_BINARY(min, NT2G_OP_MIN, false)
NT2G_BINARY(max, NT2G_OP_MAX, false)
NT2G_BINARY(adds, NT2G_OP_ADDS, false)
NT2G_BINARY(pow, NT2G_OP_POW, false)
NT2G_BINARY(atan2, NT2G_OP_ATAN2, false)
NT2G_BINARY(hypot, NT2G_OP_HYPOT, false)
NT2G_BINARY(copysign, NT2G_OP_COPYSIGN, false)
// mod(a, b) = a - floor(a/b) b, rem(a, b) = a - b itrunc(a/b) (boost/simd/arithmetic/functions/
// generic/mod.hpp, scalar/rem.hpp): a where b == 0
NT2G_BINARY(mod, NT2G_OP_MOD, false)
NT2G_BINARY(rem, NT2G_OP_REM, false)
// pow2(a, b) = a * 2^trunc(b), pow2(x) = 2^trunc(x) (EXP/generic/pow2.hpp, NT2's fast_ldexp)
NT2G_BINARY(pow2, NT2G_OP_POW2, false)
template <class A> expr<float> pow2(const A &a) { return pow2(1.0f, a); }
// nthroot(x, n), expni(n, x), gammainc(x, a), gammaincinv(p, a): the integer n is truncated
// toward zero (EXP/scalar/nthroot.hpp, EUL/scalar/expni.hpp, EUL/scalar/gammainc.hpp)
NT2G_BINARY(nthroot, NT2G_OP_NTHROOT, false)
NT2G_BINARY(expni, NT2G_OP_EXPNI, false)
NT2G_BINARY(gammainc, NT2G_OP_GAMMAINC, false)
NT2G_BINARY(gammaincinv, NT2G_OP_GAMMAINCINV, false)
#undef NT2G_BINARY

// predicates (boost/simd/predicates/functions): logical results for if_else
#define NT2G_PREDICATE(NAME, CODE)                                                                               \
    template <class A, class T = typename detail::elem_of<std::decay_t<A>>::type>                               \
    expr<T> NAME(const A &a)                                                                                     \
    {                                                                                                            \
        return expr<T>{detail::make(CODE, detail::dtype_of<T>::value, detail::lift(a)), true};                   \
    }
NT2G_PREDICATE(is_nan, NT2G_OP_IS_NAN)
NT2G_PREDICATE(is_inf, NT2G_OP_IS_INF)
NT2G_PREDICATE(is_finite, NT2G_OP_IS_FINITE)
NT2G_PREDICATE(is_eqz, NT2G_OP_IS_EQZ)
NT2G_PREDICATE(is_nez, NT2G_OP_IS_NEZ)
NT2G_PREDICATE(is_ltz, NT2G_OP_IS_LTZ)
NT2G_PREDICATE(is_gtz, NT2G_OP_IS_GTZ)
#undef NT2G_PREDICATE

#define NT2G_UNARY(NAME, CODE)                                                                                   \
    template <class A, class T = typename detail::elem_of<std::decay_t<A>>::type>                               \
    expr<T> NAME(const A &a)                                                                                     \
    {                                                                                                            \
        return expr<T>{detail::make(CODE, detail::dtype_of<T>::value, detail::lift(a))};                        \
    }

NT2G_UNARY(operator-, NT2G_OP_NEG)
NT2G_UNARY(abs, NT2G_OP_ABS)
NT2G_UNARY(sqr, NT2G_OP_SQR)
NT2G_UNARY(sqrt, NT2G_OP_SQRT)
NT2G_UNARY(rec, NT2G_OP_REC)
NT2G_UNARY(exp, NT2G_OP_EXP)
NT2G_UNARY(log, NT2G_OP_LOG)
NT2G_UNARY(log1p, NT2G_OP_LOG1P)
NT2G_UNARY(erfc, NT2G_OP_ERFC)
NT2G_UNARY(normcdf, NT2G_OP_NORMCDF)
NT2G_UNARY(fastnormcdf, NT2G_OP_FASTNORMCDF)
NT2G_UNARY(exp2, NT2G_OP_EXP2)
NT2G_UNARY(exp10, NT2G_OP_EXP10)
NT2G_UNARY(expm1, NT2G_OP_EXPM1)
NT2G_UNARY(log2, NT2G_OP_LOG2)
NT2G_UNARY(log10, NT2G_OP_LOG10)
NT2G_UNARY(sin, NT2G_OP_SIN)
NT2G_UNARY(cos, NT2G_OP_COS)
NT2G_UNARY(tan, NT2G_OP_TAN)
NT2G_UNARY(sinpi, NT2G_OP_SINPI)
NT2G_UNARY(cospi, NT2G_OP_COSPI)
NT2G_UNARY(sinh, NT2G_OP_SINH)
NT2G_UNARY(cosh, NT2G_OP_COSH)
NT2G_UNARY(tanh, NT2G_OP_TANH)
NT2G_UNARY(asin, NT2G_OP_ASIN)
NT2G_UNARY(acos, NT2G_OP_ACOS)
NT2G_UNARY(atan, NT2G_OP_ATAN)
NT2G_UNARY(asinh, NT2G_OP_ASINH)
NT2G_UNARY(acosh, NT2G_OP_ACOSH)
NT2G_UNARY(atanh, NT2G_OP_ATANH)
NT2G_UNARY(cbrt, NT2G_OP_CBRT)
NT2G_UNARY(cot, NT2G_OP_COT)
NT2G_UNARY(sec, NT2G_OP_SEC)
NT2G_UNARY(csc, NT2G_OP_CSC)
NT2G_UNARY(sind, NT2G_OP_SIND)
NT2G_UNARY(cosd, NT2G_OP_COSD)
NT2G_UNARY(tand, NT2G_OP_TAND)
NT2G_UNARY(tanpi, NT2G_OP_TANPI)
NT2G_UNARY(proper_tanpi, NT2G_OP_PROPER_TANPI)
NT2G_UNARY(cotpi, NT2G_OP_COTPI)
NT2G_UNARY(cotd, NT2G_OP_COTD)
NT2G_UNARY(secpi, NT2G_OP_SECPI)
NT2G_UNARY(cscpi, NT2G_OP_CSCPI)
NT2G_UNARY(secd, NT2G_OP_SECD)
NT2G_UNARY(cscd, NT2G_OP_CSCD)
NT2G_UNARY(sinc, NT2G_OP_SINC)
NT2G_UNARY(sincpi, NT2G_OP_SINCPI)
NT2G_UNARY(acotd, NT2G_OP_ACOTD)
NT2G_UNARY(asec, NT2G_OP_ASEC)
NT2G_UNARY(coth, NT2G_OP_COTH)
NT2G_UNARY(sinhc, NT2G_OP_SINHC)
NT2G_UNARY(acsc, NT2G_OP_ACSC)
NT2G_UNARY(asech, NT2G_OP_ASECH)
NT2G_UNARY(acoth, NT2G_OP_ACOTH)
NT2G_UNARY(acsch, NT2G_OP_ACSCH)
NT2G_UNARY(erf, NT2G_OP_ERF)
NT2G_UNARY(erfcx, NT2G_OP_ERFCX)
NT2G_UNARY(expx2, NT2G_OP_EXPX2)
NT2G_UNARY(gamma, NT2G_OP_GAMMA)
NT2G_UNARY(gammaln, NT2G_OP_GAMMALN)
NT2G_UNARY(digamma, NT2G_OP_DIGAMMA)
NT2G_UNARY(signgam, NT2G_OP_SIGNGAM)
NT2G_UNARY(dawson, NT2G_OP_DAWSON)
NT2G_UNARY(spence, NT2G_OP_SPENCE)
NT2G_UNARY(stirling, NT2G_OP_STIRLING)
NT2G_UNARY(erfinv, NT2G_OP_ERFINV)
NT2G_UNARY(erfcinv, NT2G_OP_ERFCINV)
NT2G_UNARY(floor, NT2G_OP_FLOOR)
NT2G_UNARY(ceil, NT2G_OP_CEIL)
NT2G_UNARY(trunc, NT2G_OP_TRUNC)
NT2G_UNARY(round, NT2G_OP_ROUND)
NT2G_UNARY(round2even, NT2G_OP_ROUND2EVEN)
NT2G_UNARY(frac, NT2G_OP_FRAC)
NT2G_UNARY(sign, NT2G_OP_SIGN)
NT2G_UNARY(signnz, NT2G_OP_SIGNNZ)
NT2G_UNARY(exprecneg, NT2G_OP_EXPRECNEG)
NT2G_UNARY(exprecnegc, NT2G_OP_EXPRECNEGC)
NT2G_UNARY(sqrt1pm1, NT2G_OP_SQRT1PM1)
#undef NT2G_UNARY

// NT2's generic compositions, built as the same programs of the functors
// above, operation for operation (hyperbolic/functions/generic/{sech,
// csch}.hpp; trigonometric/functions/generic/{acot,indeg,inrad,asind,acosd,
// atand,asecd,acscd,atan2d,asinpi,acospi,atanpi}.hpp)
namespace detail {
inline float f32_of_bits(std::uint32_t u)
{
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
}
}  // namespace detail

#define NT2G_COMPOSED(NAME, BODY)                                                                                \
    template <class A, class T = typename detail::elem_of<std::decay_t<A>>::type>                               \
    expr<T> NAME(const A &a)                                                                                     \
    {                                                                                                            \
        const expr<T> x{detail::lift(a)};                                                                        \
        return BODY;                                                                                             \
    }
NT2G_COMPOSED(sech, rec(cosh(x)))
NT2G_COMPOSED(csch, rec(sinh(x)))
NT2G_COMPOSED(acot, atan(rec(x)))
NT2G_COMPOSED(indeg, x * detail::f32_of_bits(0x42652ee1u) - x * detail::f32_of_bits(0xb53387c1u))
NT2G_COMPOSED(inrad, x * detail::f32_of_bits(0x3c8efa35u))
NT2G_COMPOSED(asind, indeg(asin(x)))
NT2G_COMPOSED(acosd, indeg(acos(x)))
NT2G_COMPOSED(atand, indeg(atan(x)))
NT2G_COMPOSED(asecd, indeg(asec(x)))
NT2G_COMPOSED(acscd, indeg(acsc(x)))
NT2G_COMPOSED(asinpi, detail::f32_of_bits(0x3ea2f983u) * asin(x))
NT2G_COMPOSED(acospi, detail::f32_of_bits(0x3ea2f983u) * acos(x))
NT2G_COMPOSED(atanpi, detail::f32_of_bits(0x3ea2f983u) * atan(x))
NT2G_COMPOSED(fix, trunc(x))
NT2G_COMPOSED(oneplus, x + 1.0f)
NT2G_COMPOSED(oneminus, 1.0f - x)
NT2G_COMPOSED(minusone, x - 1.0f)
NT2G_COMPOSED(sqr_abs, sqr(x))
// boost.simd's inc, dec, abss, negs and sqrs as they are for floats
// (arithmetic/functions/{generic/inc,generic/dec,generic/abss,scalar/negs,scalar/sqrs}.hpp)
NT2G_COMPOSED(inc, x + 1.0f)
NT2G_COMPOSED(dec, x - 1.0f)
NT2G_COMPOSED(abss, abs(x))
NT2G_COMPOSED(negs, -x)
NT2G_COMPOSED(sqrs, sqr(x))
#undef NT2G_COMPOSED

// dist = |a - b|, average = fma(a, 1/2, b/2) with NT2's fma (boost/simd/
// arithmetic/functions/scalar/dist.hpp, generic/average.hpp)
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> dist(const A &a, const B &b)
{
    return abs(a - b);
}
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> average(const A &a, const B &b)
{
    return fma(a, 0.5f, b * 0.5f);
}

template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> atan2d(const A &a, const B &b)
{
    return indeg(atan2(a, b));
}

// logspace_add, logspace_sub (exponential/functions/scalar/logspace_add.hpp,
// logspace_sub.hpp): log(e^a + e^b) and log(e^a - e^b) in NT2's forms; the
// real* functors are NT2's assertion-only aliases of sqrt, log and pow
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> logspace_add(const A &a, const B &b)
{
    const expr<T> x{detail::any<T>(a)}, y{detail::any<T>(b)};
    const expr<T> t = -abs(x - y);
    return if_else(t != t, x + y, max(x, y) + log1p(exp(t)));
}
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> logspace_sub(const A &a, const B &b)
{
    const expr<T> x{detail::any<T>(a)}, y{detail::any<T>(b)};
    const expr<T> d = y - x;
    return x + if_else(d > -detail::f32_of_bits(0x3f317218u), log(-expm1(d)), log1p(-exp(d)));
}
// beta and betaln (euler/functions/scalar/beta.hpp, simd/common/betaln.hpp):
// sign*exp(gammaln(a)+gammaln(b)-gammaln(y)), y = a+b, sign the product of the
// three signgam; betaln = gammaln(a)+gammaln(b)-gammaln(a+b)
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> beta(const A &a, const B &b)
{
    const expr<T> x{detail::any<T>(a)}, w{detail::any<T>(b)};
    const expr<T> y = x + w;
    return signgam(x) * signgam(w) * signgam(y) * exp(gammaln(x) + gammaln(w) - gammaln(y));
}
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> betaln(const A &a, const B &b)
{
    const expr<T> x{detail::any<T>(a)}, w{detail::any<T>(b)};
    return gammaln(x) + gammaln(w) - gammaln(x + w);
}
template <class A, class T = typename detail::elem_of<std::decay_t<A>>::type>
expr<T> realsqrt(const A &a)
{
    return sqrt(a);
}
template <class A, class T = typename detail::elem_of<std::decay_t<A>>::type>
expr<T> reallog(const A &a)
{
    return log(a);
}
template <class A, class B, class T = typename detail::common<A, B>::type>
expr<T> realpow(const A &a, const B &b)
{
    return pow(a, b);
}

// Functors on plain scalars evaluate at once, in float, with NT2's scalar
// semantics (unfused; volatile keeps the host compiler from contracting), as
// NT2's own scalar overloads do before any expression is built.
inline float sqr(float x) { volatile float r = x * x; return r; }
inline float fma(float a, float b, float c) { volatile float p = a * b; volatile float r = p + c; return r; }
inline float fnms(float a, float b, float c) { volatile float p = a * b; volatile float r = c - p; return r; }
inline float rec(float x) { return 1.0f / x; }

// fma(a,b,c) = a*b + c; fnms(a,b,c) = c - a*b  (NT2: unfused unless the fast policy)
#define NT2G_TERNARY(NAME, CODE)                                                                                 \
    template <class A, class B, class C, class T = typename detail::common3<A, B, C>::type>                     \
    expr<T> NAME(const A &a, const B &b, const C &c)                                                             \
    {                                                                                                            \
        return expr<T>{detail::make(CODE, detail::dtype_of<T>::value, detail::any<T>(a), detail::any<T>(b),    \
                                    detail::any<T>(c))};                                                         \
    }
NT2G_TERNARY(fma, NT2G_OP_FMA)
NT2G_TERNARY(fnms, NT2G_OP_FNMS)
#undef NT2G_TERNARY

template <class C, class A, class B, class T = typename detail::common<A, B>::type>
expr<T> if_else(const C &cond, const A &a, const B &b)
{
    return expr<T>{detail::make(NT2G_OP_IF_ELSE, detail::dtype_of<T>::value, detail::lift(cond), detail::any<T>(a),
                                detail::any<T>(b))};
}

template <class C, class A, class T = typename detail::elem_of<std::decay_t<A>>::type>
expr<T> selinc(const C &cond, const A &a)
{
    return expr<T>{detail::make(NT2G_OP_SELINC, detail::dtype_of<T>::value, detail::lift(cond), detail::lift(a))};
}

template <class C, class A, class T = typename detail::elem_of<std::decay_t<A>>::type>
expr<T> seldec(const C &cond, const A &a)
{
    return expr<T>{detail::make(NT2G_OP_SELDEC, detail::dtype_of<T>::value, detail::lift(cond), detail::lift(a))};
}

// ------------------------------------------------------------ generative --
// colon, linspace and logspace are expressions over the element's position p
// (NT2's enumerate<T>(p), the INDEX leaf), with NT2's sizes and values:
//   colon(l, u)     l + p, 1 x (u-l+1) elements      (generative/functions/scalar/colon.hpp:24-47,
//                                                     details/colon.hpp unity_colon_size/value)
//   colon(l, s, u)  fma(p, s, l), fuzzy element count (scalar/colon.hpp:127-160, details/colon.hpp
//                                                     colon_value; fuzzy/scalar/tolerant_floor.hpp)
//   linspace(l,u,n) p == n-1 ? u : fma(p, (u-l)/(n-1), l); n defaults to 100, n < 2 gives u
//                                                    (scalar/linspace.hpp, details/linspace.hpp)
//   logspace(l,u,n) exp10(fma(p, step, lower)), u == pi means log10(pi); n defaults to 50
//                                                    (scalar/logspace.hpp, details/logspace.hpp)
// The host-side sizes and steps use float arithmetic with every step rounded.
namespace detail {
inline float fsub(float a, float b) { volatile float r = a - b; return r; }
inline float fadd(float a, float b) { volatile float r = a + b; return r; }
inline float fmul(float a, float b) { volatile float r = a * b; return r; }
inline float fdiv(float a, float b) { volatile float r = a / b; return r; }
inline node_ptr index_leaf(std::size_t n)
{
    auto p = make(NT2G_OP_INDEX, NT2G_F32);
    p->numel = n;
    return p;
}
inline node_ptr cst(float v) { return lift_scalar<float>(v); }
inline float bits_f(std::uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
// Hagerty's FL5 tolerant floor (fuzzy/functions/scalar/tolerant_floor.hpp:33-44)
inline float tolerant_floor(float a0)
{
    const float ct = 3.0f * 1.1920929e-7f;  // Threeeps
    const float q = a0 < 0.0f ? fsub(1.0f, ct) : 1.0f;
    const float rmax = fdiv(q, fsub(2.0f, ct));
    float t1 = fadd(1.0f, std::floor(a0));
    t1 = fmul(fdiv(ct, q), t1 < 0.0f ? -t1 : t1);
    const float lo = rmax < t1 ? rmax : t1;  // NT2 min(rmax, t1) = rmax < t1 ? rmax : t1
    t1 = std::floor(fadd(a0, ct > lo ? ct : lo));
    return (a0 <= 0.0f || fsub(t1, a0) < rmax) ? t1 : fsub(t1, 1.0f);
}
inline bool fuzzy_equal(float a, float b, float tol)
{
    const float d = std::fabs(fsub(a, b));
    const float fa = std::fabs(a), fb = std::fabs(b);
    return d <= fmul(tol, fa > fb ? fa : fb);
}
inline std::size_t colon_count(float l, float s, float u)
{
    if (!s) return (std::size_t)u;
    if (!(fmul(fsub(u, l), s) >= 0.0f)) return 0;
    const std::size_t nelt = (std::size_t)tolerant_floor(fdiv(fadd(fsub(u, l), s), s));
    const float eps3 = 3.0f * 1.1920929e-7f;
    if (!fuzzy_equal(fadd(l, fmul((float)(nelt - 1), s)), u, eps3)) {
        if (fuzzy_equal(fadd(l, fmul((float)(nelt - 2), s)), u, eps3)) return nelt - 1;
        if (fuzzy_equal(fadd(l, fmul((float)nelt, s)), u, eps3)) return nelt + 1;
    }
    return nelt;
}
}  // namespace detail

inline expr<float> colon(float l, float u)
{
    const std::size_t n = u >= l ? (std::size_t)detail::fadd(detail::fsub(u, l), 1.0f) : 0;
    return expr<float>{detail::make(NT2G_OP_ADD, NT2G_F32, detail::index_leaf(n), detail::cst(l))};
}
inline expr<float> colon(float l, float s, float u)
{
    return expr<float>{detail::make(NT2G_OP_FMA, NT2G_F32, detail::index_leaf(detail::colon_count(l, s, u)),
                                    detail::cst(s), detail::cst(l))};
}
// NT2's _(l, u) / _(l, s, u) spelling of colon
struct colon_placeholder {
    expr<float> operator()(float l, float u) const { return colon(l, u); }
    expr<float> operator()(float l, float s, float u) const { return colon(l, s, u); }
};
inline constexpr colon_placeholder _{};

inline expr<float> linspace(float l, float u, std::size_t n = 100)
{
    const float lo = n < 2 ? u : l;
    const std::size_t m = n < 2 ? 2 : n;
    const float step = detail::fdiv(detail::fsub(u, lo), (float)(m - 1));
    auto p = detail::index_leaf(n);
    auto last = detail::make(NT2G_OP_EQ, NT2G_F32, p, detail::cst((float)(m - 1)));
    auto line = detail::make(NT2G_OP_FMA, NT2G_F32, p, detail::cst(step), detail::cst(lo));
    return expr<float>{detail::make(NT2G_OP_IF_ELSE, NT2G_F32, last, detail::cst(u), line)};
}
inline expr<float> logspace(float l, float u, std::size_t n = 50, bool regular = false)
{
    if (!regular && u == detail::bits_f(0x40490fdbu)) u = detail::bits_f(0x3efe8a6eu);  // Pi -> Log10_pi
    const float lower = n != 1 ? l : u;
    const float step = n != 1 ? detail::fdiv(detail::fsub(u, l), (float)(n - 1)) : 0.0f;
    auto line = detail::make(NT2G_OP_FMA, NT2G_F32, detail::index_leaf(n), detail::cst(step), detail::cst(lower));
    return expr<float>{detail::make(NT2G_OP_EXP10, NT2G_F32, line)};
}

// ones / zeros (generative/functions/{ones,zeros}.hpp): a constant table of a
// given size; ones(n) is n x n as in NT2 (and MATLAB)
inline expr<float> filled(of_size_ s, float v)
{
    auto n = detail::cst(v);
    n->numel = s.numel();
    return expr<float>{n};
}
inline expr<float> ones(of_size_ s) { return filled(s, 1.0f); }
inline expr<float> ones(std::size_t n) { return ones(of_size(n, n)); }
inline expr<float> ones(std::size_t a, std::size_t b) { return ones(of_size(a, b)); }
inline expr<float> zeros(of_size_ s) { return filled(s, 0.0f); }
inline expr<float> zeros(std::size_t n) { return zeros(of_size(n, n)); }
inline expr<float> zeros(std::size_t a, std::size_t b) { return zeros(of_size(a, b)); }

// if_zero_else_one on a logical yields the element type of the comparison
template <class T> expr<T> if_zero_else_one(const expr<T> &cond)
{
    return expr<T>{detail::make(NT2G_OP_IF_ZERO_ELSE_ONE, detail::dtype_of<T>::value, cond.n)};
}

// ------------------------------------------------------------ reductions --
namespace detail {
// Reduction scratch (workspace and result words) of the calling thread on the
// current device and stream, allocated on first use and kept for the thread's
// lifetime: no two host threads share one, a call after a device switch gets
// that device's memory, and reductions in flight on two streams never share
// one (one stream's are ordered by the stream).
struct scratch {
    device_buffer ws, out;
};
inline scratch &thread_scratch(std::size_t ws_bytes)
{
    int32_t dev = 0;
    check(nt2g_device_current(&dev), "current device");
    thread_local std::map<std::pair<int32_t, void *>, scratch> cache;
    scratch &s = cache[{dev, options().stream}];
    if (s.ws.bytes < ws_bytes) s.ws = device_buffer(ws_bytes < 256 ? 256 : ws_bytes);
    if (!s.out.p) s.out = device_buffer(64);
    return s;
}

// A table operand of a reduction as a device pointer (staged if on the host).
struct dev_view {
    const float *p = nullptr;
    std::size_t n = 0;
    device_buffer hold;
};

inline void view_of(const node *l, dev_view &v)
{
    v.n = l->numel;
    if (l->dev_ptr) { v.p = (const float *)l->dev_ptr; return; }
    if (host_in_place()) { v.p = (const float *)l->host_ptr; return; }
    v.hold = device_buffer(l->numel * sizeof(float));
    check(nt2g_memcpy(v.hold.p, l->host_ptr, l->numel * sizeof(float), 1, options().stream), "stage host table");
    v.p = (const float *)v.hold.p;
}

// The arguments of a lowered program's table leaves: device tables directly,
// host tables in place when the device reaches host memory, else staged.
inline std::vector<nt2g_arg> input_args(const lowered &L, std::vector<device_buffer> &staging)
{
    std::vector<nt2g_arg> args(L.slot_leaf.size());
    staging.reserve(L.slot_leaf.size());
    for (std::size_t s = 0; s < L.slot_leaf.size(); ++s) {
        const node *l = L.slot_leaf[s];
        nt2g_arg &a = args[s];
        a.dtype = l->dtype;
        a.kind = 0;
        a.scalar = 0.0;
        if (l->dev_ptr) a.ptr = l->dev_ptr;
        else if (host_in_place()) a.ptr = (void *)l->host_ptr;
        else {
            const std::size_t esz = l->dtype == NT2G_U8 ? 1 : 4;
            staging.emplace_back(l->numel * esz);
            a.ptr = staging.back().p;
            check(nt2g_memcpy(a.ptr, l->host_ptr, l->numel * esz, 1, options().stream), "stage host table");
        }
    }
    return args;
}

struct fold_shape {
    std::int64_t lo = 1, inner = 1, hi = 1;
};

// The fold of an expression in one pass (nt2g_eval_fold): the expression's
// value at every element is computed inside the fold kernels, NT2's fold over
// the AST itself (reduction/.../scalar/inner_fold.hpp:23-49).  out, index,
// out64 are device (or device-reachable) memory; the call is asynchronous on
// options().stream unless host tables had to be staged.
inline void fold_expr(const node_ptr &n, fold_shape f, int op, int precision, float *out, std::int64_t *index,
                      double *out64)
{
    lowering lw;
    lw.push(NT2G_OP_FOLD, NT2G_F32, lw.emit(n.get()));
    lw.finish();
    nt2g_program *prog = program_for(lw.L);
    std::vector<device_buffer> staging;
    std::vector<nt2g_arg> args = input_args(lw.L, staging);
    std::size_t b = 0;
    check(nt2g_fold_workspace_size(f.lo, f.inner, f.hi, &b), "fold workspace");
    scratch &sc = thread_scratch(b);
    check(nt2g_eval_fold(prog, args.data(), (int32_t)args.size(), f.lo, f.inner, f.hi, op, precision, sc.ws.p,
                         sc.ws.bytes, out, index, out64, options().stream),
          "fold of an expression");
    // staging buffers are released on return, and host tables read in place are the caller's again
    if (!staging.empty() || has_host_leaf(lw.L.slot_leaf))
        check(nt2g_stream_synchronize(options().stream), "fold of an expression");
}

// Element count of an expression: its table / generative leaves' (they agree).
inline std::size_t numel_of(const node_ptr &n)
{
    std::size_t numel = 0;
    std::vector<const node *> stack{n.get()};
    while (!stack.empty()) {
        const node *m = stack.back();
        stack.pop_back();
        if ((m->op == NT2G_OP_LOAD || m->op == NT2G_OP_INDEX || m->op == NT2G_OP_CONST) && m->numel)
            numel = numel ? std::min(numel, m->numel) : m->numel;
        for (const node *c : {m->a.get(), m->b.get(), m->c.get()})
            if (c) stack.push_back(c);
    }
    return numel;
}

// The FP64 sum of an expression, left on the device at *dev_result:
// sum(x) and dot(x, y) of tables through nt2g_reduce_f32, any other
// expression folded in one pass.  Elements follow options().precision (NT2's
// own arithmetic or the fast policy); the sum is the compensated one.
inline void sum_to(const node_ptr &n, double *dev_result)
{
    const bool plain = n->op == NT2G_OP_LOAD;
    const bool dot = n->op == NT2G_OP_MUL && n->a->op == NT2G_OP_LOAD && n->b->op == NT2G_OP_LOAD;
    if (plain || dot) {
        dev_view x, y;
        view_of(plain ? n.get() : n->a.get(), x);
        if (dot) view_of(n->b.get(), y);
        std::size_t b = 0;
        check(nt2g_reduce_workspace_size((int64_t)x.n, &b), "reduce workspace");
        scratch &sc = thread_scratch(b);
        check(nt2g_reduce_f32(x.p, dot ? y.p : nullptr, (int64_t)x.n, sc.ws.p, sc.ws.bytes, dev_result, nullptr,
                              options().stream),
              "reduce");
        // staging buffers are released on return, host tables read in place are the caller's again
        const bool host = !(plain ? n : n->a)->dev_ptr || (dot && !n->b->dev_ptr);
        if (host) check(nt2g_stream_synchronize(options().stream), "reduce");
        return;
    }
    const std::int64_t numel = (std::int64_t)numel_of(n);
    const int prec = options().precision == NT2G_PREC_NT2 ? NT2G_PREC_NT2_ELEMENTS : NT2G_PREC_FAST;
    scratch &sc = thread_scratch(0);
    fold_expr(n, fold_shape{1, numel, 1}, NT2G_FOLD_SUM, prec, (float *)((char *)sc.out.p + 32), nullptr, dev_result);
}

inline double sum_node(const node_ptr &n)
{
    scratch &sc = thread_scratch(0);
    double *d = (double *)sc.out.p;
    sum_to(n, d);
    double r = 0;
    check(nt2g_memcpy(&r, d, sizeof r, 2, options().stream), "reduce result");
    check(nt2g_stream_synchronize(options().stream), "reduce result");
    return r;
}
}  // namespace detail

// Distribution functions of NT2's statistics module as NT2 composes them
// (modules/core/statistics/include/nt2/statistics/functions/generic/{norm,exp,logn,unif,cau,ev}{pdf,cdf,inv}.hpp),
// every operation in NT2's order; parameters are floats or expressions.
// if_zero_else(c, x) = c ? 0 : x, if_allbits_else(c, x) = c ? NaN : x,
// is_not_greater(a, b) = !(a > b), is_negative = the sign bit.
namespace detail {
inline float stat_c(std::uint32_t b) { return f32_of_bits(b); }
constexpr std::uint32_t kInvsqrt2pi = 0x3ecc422au, kSqrt2 = 0x3fb504f3u, kSqrt2o2 = 0x3f3504f3u, kInvpi = 0x3ea2f983u;
template <class X> expr<float> lift_expr(const X &x) { return expr<float>{lift(x)}; }
inline expr<float> as_expr(float v) { return expr<float>{any<float>(v)}; }
inline expr<float> as_expr(const expr<float> &e) { return e; }
// a select on a condition known on the host (parameters given as numbers) or per element
template <class A, class B> expr<float> sel(bool c, const A &a, const B &b) { return c ? as_expr(a) : as_expr(b); }
template <class T, class A, class B> expr<float> sel(const expr<T> &c, const A &a, const B &b)
{
    return if_else(c, as_expr(a), as_expr(b));
}
}  // namespace detail
template <class X> expr<float> normpdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return exp(-0.5f * sqr(a)) * detail::stat_c(detail::kInvsqrt2pi);
}
template <class X, class M> expr<float> normpdf(const X &x, const M &m)
{
    const expr<float> a{detail::lift(x)};
    return exp(-0.5f * sqr(a - m)) * detail::stat_c(detail::kInvsqrt2pi);
}
template <class X, class M, class S> expr<float> normpdf(const X &x, const M &m, const S &s)
{
    const expr<float> a{detail::lift(x)};
    const auto inv = 1.0f / s;
    return exp(-0.5f * sqr((a - m) * inv)) * detail::stat_c(detail::kInvsqrt2pi) * inv;
}
template <class X> expr<float> norminv(const X &p)
{
    const expr<float> a{detail::lift(p)};
    return -detail::stat_c(detail::kSqrt2) * erfcinv(2.0f * a);
}
template <class X, class M> expr<float> norminv(const X &p, const M &m) { return norminv(p) + m; }
template <class X, class M, class S> expr<float> norminv(const X &p, const M &m, const S &s)
{
    return fma(norminv(p), s, m);
}
template <class X> expr<float> expcdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return -expm1(-detail::sel(is_ltz(a), 0.0f, a));
}
template <class X, class M> expr<float> expcdf(const X &x, const M &mu) { return expcdf(detail::lift_expr(x) / mu); }
template <class X> expr<float> exppdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return detail::sel(is_ltz(a), 0.0f, exp(-a));
}
template <class X, class L> expr<float> exppdf(const X &x, const L &l)
{
    const expr<float> a{detail::lift(x)};
    return detail::sel(is_ltz(a), 0.0f, l * exp(-a * l));
}
template <class X> expr<float> expinv(const X &p)
{
    const expr<float> a{detail::lift(p)};
    return detail::sel(is_ltz(a), NAN, -log1p(-a));
}
template <class X, class M> expr<float> expinv(const X &p, const M &mu) { return mu * expinv(p); }
template <class X> expr<float> logncdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return 0.5f * erfc(-detail::stat_c(detail::kSqrt2o2) * log(detail::sel(a <= 0.0f, 0.0f, a)));
}
template <class X, class M> expr<float> logncdf(const X &x, const M &m)
{
    const expr<float> a{detail::lift(x)};
    return 0.5f * erfc(detail::stat_c(detail::kSqrt2o2) * (m - log(detail::sel(a <= 0.0f, 0.0f, a))));
}
template <class X, class M, class S> expr<float> logncdf(const X &x, const M &m, const S &s)
{
    const expr<float> a{detail::lift(x)};
    return 0.5f * erfc(detail::stat_c(detail::kSqrt2o2) * ((m - log(detail::sel(a <= 0.0f, 0.0f, a))) / s));
}
template <class X> expr<float> lognpdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    const expr<float> xx = detail::sel(a <= 0.0f, INFINITY, a);
    return normpdf(log(xx)) / xx;
}
template <class X, class M> expr<float> lognpdf(const X &x, const M &m)
{
    const expr<float> a{detail::lift(x)};
    const expr<float> xx = detail::sel(a <= 0.0f, INFINITY, a);
    return normpdf(log(xx), m) / xx;
}
template <class X, class M, class S> expr<float> lognpdf(const X &x, const M &m, const S &s)
{
    const expr<float> a{detail::lift(x)};
    const expr<float> xx = detail::sel(a <= 0.0f, INFINITY, a);
    return normpdf(log(xx), m, s) / xx;
}
template <class X> expr<float> logninv(const X &p)
{
    const expr<float> a{detail::lift(p)};
    return exp(-detail::stat_c(detail::kSqrt2) * erfcinv(2.0f * a));
}
template <class X, class M> expr<float> logninv(const X &p, const M &m)
{
    const expr<float> a{detail::lift(p)};
    return exp(-detail::stat_c(detail::kSqrt2) * erfcinv(2.0f * a) + m);
}
template <class X, class M, class S> expr<float> logninv(const X &p, const M &m, const S &s)
{
    const expr<float> a{detail::lift(p)};
    return exp(-detail::stat_c(detail::kSqrt2) * s * erfcinv(2.0f * a) + m);
}
template <class X> expr<float> unifcdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return detail::sel(is_ltz(a), 0.0f, detail::sel(a > 1.0f, 1.0f, a));
}
template <class X, class A, class B> expr<float> unifcdf(const X &x, const A &lo, const B &hi)
{
    const expr<float> a{detail::lift(x)};
    const auto z = hi - lo;
    return detail::sel(z <= 0.0f, NAN, detail::sel(a < lo, 0.0f, detail::sel(a > hi, 1.0f, (a - lo) / z)));
}
template <class X> expr<float> unifpdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return detail::sel(is_nan(a), a, detail::sel(a <= 1.0f, detail::sel(copysign(1.0f, a) < 0.0f, 0.0f, 1.0f), 0.0f));
}
template <class X> expr<float> unifinv(const X &p)
{
    const expr<float> a{detail::lift(p)};
    return detail::sel(a < 0.0f, NAN, detail::sel(a <= 1.0f, a, NAN));
}
template <class X, class M, class S> expr<float> caucdf(const X &x, const M &m, const S &s)
{
    const expr<float> a{detail::lift(x)};
    return 0.5f + atanpi((a - m) / s);
}
template <class X> expr<float> caucdf(const X &x) { return 0.5f + atanpi(detail::lift_expr(x)); }
template <class X, class M> expr<float> caucdf(const X &x, const M &m) { return caucdf(detail::lift_expr(x) - m); }
// boost.simd's NaN-ignoring and magnitude selects, minmod, negate, fms and
// fnma as their scalar float definitions compose them
// (boost/simd/ieee/functions/scalar/{maxnum,minnum,maxmag,minmag,negate}.hpp,
// boost/simd/arithmetic/functions/{scalar/minmod,generic/fms,generic/fnma}.hpp)
// boost.simd's rounded quotients for floats (boost/simd/arithmetic/functions/
// scalar/{divfloor,divceil,divfix,divround,divround2even}.hpp): the rounding of
// the correctly rounded a/b
template <class A, class B> expr<float> divfloor(const A &a, const B &b) { return floor(detail::lift_expr(a) / b); }
template <class A, class B> expr<float> divceil(const A &a, const B &b) { return ceil(detail::lift_expr(a) / b); }
template <class A, class B> expr<float> divfix(const A &a, const B &b) { return trunc(detail::lift_expr(a) / b); }
template <class A, class B> expr<float> divround(const A &a, const B &b) { return round(detail::lift_expr(a) / b); }
template <class A, class B> expr<float> divround2even(const A &a, const B &b)
{
    return round2even(detail::lift_expr(a) / b);
}
template <class A, class B> expr<float> maxnum(const A &a, const B &b)
{
    return if_else(is_nan(detail::lift_expr(a)), b, max(b, a));
}
template <class A, class B> expr<float> minnum(const A &a, const B &b)
{
    return if_else(is_nan(detail::lift_expr(a)), b, min(b, a));
}
template <class A, class B> expr<float> maxmag(const A &a, const B &b)
{
    const expr<float> x = detail::lift_expr(a), y = detail::lift_expr(b);
    return if_else(abs(x) > abs(y), x, if_else(abs(y) > abs(x), y, max(x, y)));
}
template <class A, class B> expr<float> minmag(const A &a, const B &b)
{
    const expr<float> x = detail::lift_expr(a), y = detail::lift_expr(b);
    return if_else(abs(x) < abs(y), x, if_else(abs(y) < abs(x), y, min(x, y)));
}
template <class A, class B> expr<float> minmod(const A &a, const B &b)
{
    const expr<float> x = detail::lift_expr(a), y = detail::lift_expr(b);
    return if_else(x * y < 0.0f, 0.0f, min(x, y));
}
template <class A, class B> expr<float> negate(const A &a, const B &b)
{
    return detail::lift_expr(a) * sign(detail::lift_expr(b));
}
template <class A, class B, class C> expr<float> fms(const A &a, const B &b, const C &c)
{
    return detail::lift_expr(a) * b - c;
}
template <class A, class B, class C> expr<float> fnma(const A &a, const B &b, const C &c)
{
    return -detail::lift_expr(c) - detail::lift_expr(a) * b;
}

template <class X> expr<float> cauinv(const X &p) { return proper_tanpi(detail::lift_expr(p) - 0.5f); }
template <class X, class M> expr<float> cauinv(const X &p, const M &m) { return cauinv(p) + m; }
template <class X, class M, class S> expr<float> cauinv(const X &p, const M &m, const S &s)
{
    return fma(cauinv(p), s, m);
}
template <class X> expr<float> caupdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    return rec(1.0f + sqr(a)) * detail::stat_c(detail::kInvpi);
}
template <class X, class M> expr<float> caupdf(const X &x, const M &m) { return caupdf(detail::lift_expr(x) - m); }
template <class X, class M, class S> expr<float> caupdf(const X &x, const M &m, const S &s)
{
    const expr<float> a{detail::lift(x)};
    return (s * detail::stat_c(detail::kInvpi)) / (s * s + sqr(a - m));
}
template <class X> expr<float> evcdf(const X &x) { return -expm1(-exp(detail::lift_expr(x))); }
template <class X, class M> expr<float> evcdf(const X &x, const M &m) { return evcdf(detail::lift_expr(x) - m); }
template <class X, class M, class S> expr<float> evcdf(const X &x, const M &m, const S &s)
{
    return evcdf((detail::lift_expr(x) - m) / s);
}
template <class X> expr<float> evpdf(const X &x)
{
    const expr<float> a{detail::lift(x)};
    const expr<float> t = exp(a);
    return detail::sel(a == INFINITY, 0.0f, t * exp(-t));
}
template <class X, class M> expr<float> evpdf(const X &x, const M &m)
{
    const expr<float> a{detail::lift(x)};
    const expr<float> t = exp(a - m);
    return detail::sel(a == INFINITY, 0.0f, t * exp(-t));
}
template <class X, class M, class S> expr<float> evpdf(const X &x, const M &m, const S &s)
{
    const expr<float> a{detail::lift(x)};
    const auto inv = 1.0f / s;
    const expr<float> t = exp((a - m) * inv);
    return detail::sel(a == INFINITY, 0.0f, t * (exp(-t) * inv));
}
template <class X> expr<float> evinv(const X &p)
{
    const expr<float> a{detail::lift(p)};
    return log(-log1p(-a));
}
template <class X, class M> expr<float> evinv(const X &p, const M &m) { return evinv(p) + m; }
template <class X, class M, class S> expr<float> evinv(const X &p, const M &m, const S &s)
{
    return evinv(p) * s + m;
}

// NT2's sum over a vector / globalsum: the compensated device reduction,
// returned as T (NT2's result type) -- sum64 keeps the FP64 combine.  A sum of
// an expression (sum(exp(x)*y), globalsum(a*b+c)) is folded in one pass, the
// expression evaluated inside the fold: no temporary table.
template <class X> double sum64(const X &x) { return detail::sum_node(detail::lift(x)); }
template <class X> float sum(const X &x) { return (float)sum64(x); }
template <class X> float globalsum(const X &x) { return (float)sum64(x); }
template <class A, class B> float dot(const A &a, const B &b) { return (float)sum64(a * b); }
// sum64 without a host round trip: the FP64 result is written to dev_result
// (device or device-reachable memory) in stream order on options().stream;
// read it after synchronizing that stream.
template <class X> void sum64_async(const X &x, double *dev_result) { detail::sum_to(detail::lift(x), dev_result); }

// ------------------------------------------------ reductions along a dimension --
// sum(a, dim), prod, maximum, minimum, mean, asum1, asum2, norm2 of a float
// table, as NT2 folds them: the extent split into [lo, inner, hi] around dim
// (core/reduction/include/nt2/dsl/functions/reduction/run.hpp:51-89), the result
// a table of the same site with extent 1 along dim.  The global forms fold the
// whole table.  options().precision selects NT2's in-order fold (NT2G_PREC_NT2)
// or the compensated one.
namespace detail {
inline fold_shape split(const of_size_ &e, int dim)
{
    fold_shape f;
    for (int k = 0; k < 4; ++k) {
        if (k < dim - 1) f.lo *= (std::int64_t)e.d[k];
        else if (k == dim - 1) f.inner = (std::int64_t)e.d[k];
        else f.hi *= (std::int64_t)e.d[k];
    }
    return f;
}
// NT2's default reduction dimension: the first non-singleton one
inline int first_non_singleton(const of_size_ &e)
{
    for (int k = 0; k < 4; ++k)
        if (e.d[k] != 1) return k + 1;
    return 1;
}
// fold x (device pointer, or host memory the device reaches) into out / index;
// host: x or out is host memory, which the caller may read or free as soon as
// the call returns (the fold is then waited for)
inline void fold_raw(const float *x, fold_shape f, int op, float *out, std::int64_t *index, bool host)
{
    std::size_t b = 0;
    check(nt2g_fold_workspace_size(f.lo, f.inner, f.hi, &b), "fold workspace");
    scratch &sc = thread_scratch(b);
    check(nt2g_fold_f32(x, f.lo, f.inner, f.hi, op, options().precision, sc.ws.p, sc.ws.bytes, out, index,
                        options().stream),
          "fold");
    if (host) check(nt2g_stream_synchronize(options().stream), "fold");
}
template <class Site>
inline table<float, Site> fold_dim(const table<float, Site> &t, int dim, int op)
{
    if (dim < 1 || dim > 4) throw gpu_error(NT2G_ERR_INVALID, "reduction dimension out of range");
    of_size_ e = t.extent();
    const fold_shape f = split(e, dim);
    e.d[dim - 1] = 1;
    table<float, Site> r(e);
    const bool direct = table<float, Site>::on_device || host_in_place();
    if (direct) {
        fold_raw(t.data(), f, op, r.data(), nullptr, !table<float, Site>::on_device);
    } else {  // host tables the device cannot reach: through device buffers
        table<float, device_> dt(t.extent()), dr(e);
        dt = t;
        fold_raw(dt.data(), f, op, dr.data(), nullptr, false);
        r = dr;
    }
    return r;
}
template <class Site>
inline float fold_all(const table<float, Site> &t, int op, std::int64_t *index1 = nullptr)
{
    const fold_shape f{1, (std::int64_t)t.numel(), 1};
    scratch &sc = thread_scratch(0);  // the float result at 16, the int64 position at 24
    float *o = (float *)((char *)sc.out.p + 16);
    std::int64_t *ix = index1 ? (std::int64_t *)((char *)sc.out.p + 24) : nullptr;
    if (table<float, Site>::on_device || host_in_place()) {
        fold_raw(t.data(), f, op, o, ix, false);  // waited for below
    } else {
        table<float, device_> dt(t.extent());
        dt = t;
        fold_raw(dt.data(), f, op, o, ix, false);
    }
    float r = 0.0f;
    check(nt2g_memcpy(&r, o, sizeof r, 2, options().stream), "fold result");
    if (ix) {
        check(nt2g_memcpy(index1, ix, sizeof *ix, 2, options().stream), "fold index");
        *index1 += 1;  // NT2 positions are 1-based (0: none)
    }
    check(nt2g_stream_synchronize(options().stream), "fold result");
    return r;
}

// Folds of an expression (one pass, no temporary).  Its extent is its first
// table leaf's (a row of numel elements when it has only generative leaves).
inline of_size_ extent_of(const node_ptr &n)
{
    std::vector<const node *> stack{n.get()};
    while (!stack.empty()) {
        const node *m = stack.back();
        stack.pop_back();
        if (m->op == NT2G_OP_LOAD && m->ext[0]) return of_size(m->ext[0], m->ext[1], m->ext[2], m->ext[3]);
        for (const node *c : {m->c.get(), m->b.get(), m->a.get()})
            if (c) stack.push_back(c);
    }
    return of_size(1, numel_of(n));
}
inline table<float, device_> fold_dim_expr(const node_ptr &n, int dim, int op)
{
    if (dim < 1 || dim > 4) throw gpu_error(NT2G_ERR_INVALID, "reduction dimension out of range");
    of_size_ e = extent_of(n);
    const fold_shape f = split(e, dim);
    e.d[dim - 1] = 1;
    table<float, device_> r(e);
    fold_expr(n, f, op, options().precision, r.data(), nullptr, nullptr);
    return r;
}
inline float fold_all_expr(const node_ptr &n, int op, std::int64_t *index1 = nullptr)
{
    scratch &sc = thread_scratch(0);
    float *o = (float *)((char *)sc.out.p + 16);
    std::int64_t *ix = index1 ? (std::int64_t *)((char *)sc.out.p + 24) : nullptr;
    fold_expr(n, fold_shape{1, (std::int64_t)numel_of(n), 1}, op, options().precision, o, ix, nullptr);
    float r = 0.0f;
    check(nt2g_memcpy(&r, o, sizeof r, 2, options().stream), "fold result");
    if (ix) {
        check(nt2g_memcpy(index1, ix, sizeof *ix, 2, options().stream), "fold index");
        *index1 += 1;  // NT2 positions are 1-based (0: none)
    }
    check(nt2g_stream_synchronize(options().stream), "fold result");
    return r;
}
}  // namespace detail

// The reductions of an expression: sum(exp(x)*y, 1), maximum(abs(a - b), 2),
// globalmax(a*b + c), ... fold the expression in one pass (the tables are read
// once, no temporary), as NT2's folds take the expression itself.  The result
// of a reduction along a dimension is a device table.
#define NT2G_EXPR_FOLD(NAME, OP)                                                                           \
    template <class T> table<float, device_> NAME(const expr<T> &e, int dim)                                \
    {                                                                                                       \
        return detail::fold_dim_expr(e.n, dim, OP);                                                         \
    }
NT2G_EXPR_FOLD(sum, NT2G_FOLD_SUM)
NT2G_EXPR_FOLD(prod, NT2G_FOLD_PROD)
NT2G_EXPR_FOLD(maximum, NT2G_FOLD_MAX)
NT2G_EXPR_FOLD(minimum, NT2G_FOLD_MIN)
NT2G_EXPR_FOLD(mean, NT2G_FOLD_MEAN)
NT2G_EXPR_FOLD(asum1, NT2G_FOLD_ASUM1)
NT2G_EXPR_FOLD(asum2, NT2G_FOLD_ASUM2)
NT2G_EXPR_FOLD(norm2, NT2G_FOLD_NORM2)
NT2G_EXPR_FOLD(nbtrue, NT2G_FOLD_NBTRUE)
NT2G_EXPR_FOLD(nansum, NT2G_FOLD_NANSUM)
#undef NT2G_EXPR_FOLD
#define NT2G_EXPR_GLOBAL(NAME, OP)                                                                         \
    template <class T> float NAME(const expr<T> &e) { return detail::fold_all_expr(e.n, OP); }
NT2G_EXPR_GLOBAL(globalmax, NT2G_FOLD_MAX)
NT2G_EXPR_GLOBAL(globalmin, NT2G_FOLD_MIN)
NT2G_EXPR_GLOBAL(globalprod, NT2G_FOLD_PROD)
NT2G_EXPR_GLOBAL(globalmean, NT2G_FOLD_MEAN)
NT2G_EXPR_GLOBAL(globalasum1, NT2G_FOLD_ASUM1)
NT2G_EXPR_GLOBAL(globalasum2, NT2G_FOLD_ASUM2)
NT2G_EXPR_GLOBAL(globalnorm2, NT2G_FOLD_NORM2)
NT2G_EXPR_GLOBAL(globalnbtrue, NT2G_FOLD_NBTRUE)
NT2G_EXPR_GLOBAL(globalnansum, NT2G_FOLD_NANSUM)
NT2G_EXPR_GLOBAL(globalnanmean, NT2G_FOLD_NANMEAN)
#undef NT2G_EXPR_GLOBAL
template <class T> float globalmax(const expr<T> &e, std::int64_t &i) { return detail::fold_all_expr(e.n, NT2G_FOLD_MAX, &i); }
template <class T> float globalmin(const expr<T> &e, std::int64_t &i) { return detail::fold_all_expr(e.n, NT2G_FOLD_MIN, &i); }
template <class T> float globalvar(const expr<T> &e, int w = 0)
{
    return detail::fold_all_expr(e.n, w ? NT2G_FOLD_VAR1 : NT2G_FOLD_VAR);
}
template <class T> float globalstdev(const expr<T> &e, int w = 0)
{
    return detail::fold_all_expr(e.n, w ? NT2G_FOLD_STDEV1 : NT2G_FOLD_STDEV);
}
template <class T> table<float, device_> var(const expr<T> &e, int w, int dim)
{
    return detail::fold_dim_expr(e.n, dim, w ? NT2G_FOLD_VAR1 : NT2G_FOLD_VAR);
}
template <class T> table<float, device_> stdev(const expr<T> &e, int w, int dim)
{
    return detail::fold_dim_expr(e.n, dim, w ? NT2G_FOLD_STDEV1 : NT2G_FOLD_STDEV);
}

#define NT2G_DIM_FOLD(NAME, OP)                                                                            \
    template <class Site> table<float, Site> NAME(const table<float, Site> &t, int dim)                     \
    {                                                                                                       \
        return detail::fold_dim(t, dim, OP);                                                                \
    }
NT2G_DIM_FOLD(sum, NT2G_FOLD_SUM)
NT2G_DIM_FOLD(prod, NT2G_FOLD_PROD)
NT2G_DIM_FOLD(maximum, NT2G_FOLD_MAX)
NT2G_DIM_FOLD(minimum, NT2G_FOLD_MIN)
NT2G_DIM_FOLD(mean, NT2G_FOLD_MEAN)
NT2G_DIM_FOLD(asum1, NT2G_FOLD_ASUM1)
NT2G_DIM_FOLD(asum2, NT2G_FOLD_ASUM2)
NT2G_DIM_FOLD(norm2, NT2G_FOLD_NORM2)
#undef NT2G_DIM_FOLD

// var(t, w, dim), stdev(t, w, dim) (reduction/functions/expr/{var,stdev}.hpp):
// w = 0 divides by n - 1, w = 1 by n
template <class Site> table<float, Site> var(const table<float, Site> &t, int w, int dim)
{
    return detail::fold_dim(t, dim, w ? NT2G_FOLD_VAR1 : NT2G_FOLD_VAR);
}
template <class Site> table<float, Site> stdev(const table<float, Site> &t, int w, int dim)
{
    return detail::fold_dim(t, dim, w ? NT2G_FOLD_STDEV1 : NT2G_FOLD_STDEV);
}
// nbtrue, all, any, none along a dimension (nonzero elements, NaN included);
// nansum and nanmean (reduction/functions/expr/{nansum,nanmean}.hpp)
#define NT2G_DIM_FOLD(NAME, OP)                                                                            \
    template <class Site> table<float, Site> NAME(const table<float, Site> &t, int dim)                     \
    {                                                                                                       \
        return detail::fold_dim(t, dim, OP);                                                                \
    }                                                                                                       \
    template <class Site> table<float, Site> NAME(const table<float, Site> &t)                              \
    {                                                                                                       \
        return detail::fold_dim(t, detail::first_non_singleton(t.extent()), OP);                            \
    }
NT2G_DIM_FOLD(nbtrue, NT2G_FOLD_NBTRUE)
NT2G_DIM_FOLD(all, NT2G_FOLD_ALL)
NT2G_DIM_FOLD(any, NT2G_FOLD_ANY)
NT2G_DIM_FOLD(none, NT2G_FOLD_NONE)
NT2G_DIM_FOLD(nansum, NT2G_FOLD_NANSUM)
NT2G_DIM_FOLD(nanmean, NT2G_FOLD_NANMEAN)
NT2G_DIM_FOLD(meanad, NT2G_FOLD_MEANAD)  // mean(abs(center(t, dim)), dim) (reduction/functions/expr/meanad.hpp)
#undef NT2G_DIM_FOLD

// wmean(t, w[, dim]) (reduction/functions/expr/wmean.hpp): rec(globalsum(w))
// times sum(t .* w, dim), the product folded in one pass
template <class Site> table<float, device_> wmean(const table<float, Site> &t, const table<float, Site> &w, int dim)
{
    const float f = 1.0f / globalsum(w);
    const table<float, device_> s = sum(t * w, dim);
    table<float, device_> r(s.extent());
    r = f * s;
    return r;
}
template <class Site> table<float, device_> wmean(const table<float, Site> &t, const table<float, Site> &w)
{
    return wmean(t, w, detail::first_non_singleton(t.extent()));
}

// asump(t, p[, dim]) = sum(pow_abs(t, p), dim) and normp(t, p[, dim]) =
// pow(asump, rec(p)) (core/functions/expr/asump.hpp:17-49, normp.hpp:17-49);
// NT2's pow_abs(a, p) is its pow of the non-negative |a|, so the fold takes
// pow(abs(t), p) in one pass.  globalasump / globalnormp fold every element
// (globalasump is a global sum, the compensated reduction; NT2's pow of the
// result is evaluated on the device).
template <class Site> table<float, device_> asump(const table<float, Site> &t, float p, int dim)
{
    return sum(pow(abs(t), p), dim);
}
template <class Site> table<float, device_> asump(const table<float, Site> &t, float p)
{
    return asump(t, p, detail::first_non_singleton(t.extent()));
}
template <class Site> table<float, device_> normp(const table<float, Site> &t, float p, int dim)
{
    const table<float, device_> s = asump(t, p, dim);
    table<float, device_> r(s.extent());
    r = pow(s, 1.0f / p);
    return r;
}
template <class Site> table<float, device_> normp(const table<float, Site> &t, float p)
{
    return normp(t, p, detail::first_non_singleton(t.extent()));
}
template <class Site> float globalasump(const table<float, Site> &t, float p) { return globalsum(pow(abs(t), p)); }
template <class Site> float globalnormp(const table<float, Site> &t, float p)
{
    table<float> h(of_size(1));
    h(1) = globalasump(t, p);
    table<float> r(of_size(1));
    r = pow(h, 1.0f / p);
    return r(1);
}

template <class Site> table<float, Site> var(const table<float, Site> &t, int w = 0)
{
    return var(t, w, detail::first_non_singleton(t.extent()));
}
template <class Site> table<float, Site> stdev(const table<float, Site> &t, int w = 0)
{
    return stdev(t, w, detail::first_non_singleton(t.extent()));
}

template <class Site> float globalmax(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_MAX); }
template <class Site> float globalmin(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_MIN); }
// globalmax(t, i): i receives the 1-based linear position of the first element equal to the maximum
template <class Site> float globalmax(const table<float, Site> &t, std::int64_t &i)
{
    return detail::fold_all(t, NT2G_FOLD_MAX, &i);
}
template <class Site> float globalmin(const table<float, Site> &t, std::int64_t &i)
{
    return detail::fold_all(t, NT2G_FOLD_MIN, &i);
}
template <class Site> float globalprod(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_PROD); }
template <class Site> float globalmean(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_MEAN); }
template <class Site> float globalasum1(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_ASUM1); }
template <class Site> float globalasum2(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_ASUM2); }
template <class Site> float globalnorm2(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_NORM2); }
template <class Site> bool globalall(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_ALL) != 0.0f; }
template <class Site> bool globalany(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_ANY) != 0.0f; }
template <class Site> bool globalnone(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_NONE) != 0.0f; }
template <class Site> float globalnbtrue(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_NBTRUE); }
template <class Site> float globalnansum(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_NANSUM); }
template <class Site> float globalnanmean(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_NANMEAN); }
template <class Site> float globalvar(const table<float, Site> &t, int w = 0)
{
    return detail::fold_all(t, w ? NT2G_FOLD_VAR1 : NT2G_FOLD_VAR);
}
template <class Site> float globalstdev(const table<float, Site> &t, int w = 0)
{
    return detail::fold_all(t, w ? NT2G_FOLD_STDEV1 : NT2G_FOLD_STDEV);
}
// globalmeanad(t) = meanad(t(:)) (core/functions/globalmeanad.hpp)
template <class Site> float globalmeanad(const table<float, Site> &t) { return detail::fold_all(t, NT2G_FOLD_MEANAD); }
// nanasum2(t[, dim]) = sum(if_zero_else(is_nan(t), sqr_abs(t)), dim)
// (core/functions/expr/nanasum2.hpp), folded in one pass
template <class Site> table<float, device_> nanasum2(const table<float, Site> &t, int dim)
{
    return sum(if_else(is_nan(t), 0.0f, t * t), dim);
}
template <class Site> table<float, device_> nanasum2(const table<float, Site> &t)
{
    return nanasum2(t, detail::first_non_singleton(t.extent()));
}
// globalnorm(t[, p]) (core/functions/expr/globalnorm.hpp): globalnorm2 by
// default and for p = 2, globalasum1 for p = 1, the largest / smallest |t|
// for p = +inf / -inf, else globalnormp(t, p)
template <class Site> float globalnorm(const table<float, Site> &t, float p = 2.0f)
{
    if (p == 2.0f) return globalnorm2(t);
    if (p == 1.0f) return globalasum1(t);
    if (p == INFINITY || p == -INFINITY) {
        table<float, device_> a(t.extent());
        a = abs(t);
        return p > 0 ? globalmax(a) : globalmin(a);
    }
    return globalnormp(t, p);
}
// cumsum(t, dim), cumprod, cummax, cummin: tables of the shape of t
namespace detail {
template <class Site> inline table<float, Site> scan_dim(const table<float, Site> &t, int dim, int op)
{
    if (dim < 1 || dim > 4) throw gpu_error(NT2G_ERR_INVALID, "cumulative dimension out of range");
    const fold_shape f = split(t.extent(), dim);
    table<float, Site> r(t.extent());
    auto run = [&](const float *x, float *o) {
        std::size_t b = 0;
        check(nt2g_scan_workspace_size(f.lo, f.inner, f.hi, &b), "scan workspace");
        scratch &sc = thread_scratch(b);
        check(nt2g_scan_f32(x, f.lo, f.inner, f.hi, op, options().precision, sc.ws.p, sc.ws.bytes, o,
                            options().stream),
              "scan");
        // a host table read or written in place is the caller's as soon as this returns
        if (!table<float, Site>::on_device) check(nt2g_stream_synchronize(options().stream), "scan");
    };
    if (table<float, Site>::on_device || host_in_place()) {
        run(t.data(), r.data());
    } else {
        table<float, device_> dt(t.extent()), dr(t.extent());
        dt = t;
        run(dt.data(), dr.data());
        r = dr;
    }
    return r;
}
}  // namespace detail
// median(t, dim), medianad(t, dim) (core/functions/expr/median.hpp,
// expr/medianad.hpp): the middle element of each slice along dim (meanof
// of the two middle ones for an even length), by selection on the device;
// globalmedian / globalmedianad over all elements.
namespace detail {
template <class Site> inline void median_raw(const table<float, Site> &t, fold_shape f, int op, float *o)
{
    auto run = [&](const float *x) {
        std::size_t b = 0;
        check(nt2g_median_workspace_size(f.lo, f.inner, f.hi, &b), "median workspace");
        scratch &sc = thread_scratch(b);
        check(nt2g_median_f32(x, f.lo, f.inner, f.hi, op, sc.ws.p, sc.ws.bytes, o, options().stream), "median");
        if (!table<float, Site>::on_device) check(nt2g_stream_synchronize(options().stream), "median");
    };
    if (table<float, Site>::on_device || host_in_place()) {
        run(t.data());
    } else {
        table<float, device_> dt(t.extent());
        dt = t;
        run(dt.data());
    }
}
template <class Site> inline table<float, device_> median_dim(const table<float, Site> &t, int dim, int op)
{
    if (dim < 1 || dim > 4) throw gpu_error(NT2G_ERR_INVALID, "median dimension out of range");
    of_size_ e = t.extent();
    const fold_shape f = split(e, dim);
    e.d[dim - 1] = 1;
    table<float, device_> r(e);
    median_raw(t, f, op, r.data());
    return r;
}
template <class Site> inline float median_all(const table<float, Site> &t, int op)
{
    scratch &sc = thread_scratch(0);
    float *o = (float *)((char *)sc.out.p + 16);
    median_raw(t, fold_shape{1, (std::int64_t)t.numel(), 1}, op, o);
    float r = 0.0f;
    check(nt2g_memcpy(&r, o, sizeof r, 2, options().stream), "median result");
    check(nt2g_stream_synchronize(options().stream), "median result");
    return r;
}
}  // namespace detail
// trapz(t[, dim]) (core/functions/expr/trapz.hpp): half the sum of the sums
// of neighbours along dim (unit spacing)
template <class Site> table<float, device_> trapz(const table<float, Site> &t, int dim)
{
    if (dim < 1 || dim > 4) throw gpu_error(NT2G_ERR_INVALID, "trapz dimension out of range");
    of_size_ e = t.extent();
    const detail::fold_shape f = detail::split(e, dim);
    e.d[dim - 1] = 1;
    table<float, device_> r(e);
    auto run = [&](const float *x) {
        std::size_t b = 0;
        check(nt2g_trapz_workspace_size(f.lo, f.inner, f.hi, &b), "trapz workspace");
        detail::scratch &sc = detail::thread_scratch(b);
        check(nt2g_trapz_f32(x, f.lo, f.inner, f.hi, options().precision, sc.ws.p, sc.ws.bytes, r.data(),
                             options().stream),
              "trapz");
        if (!table<float, Site>::on_device) check(nt2g_stream_synchronize(options().stream), "trapz");
    };
    if (table<float, Site>::on_device || detail::host_in_place()) {
        run(t.data());
    } else {
        table<float, device_> dt(t.extent());
        dt = t;
        run(dt.data());
    }
    return r;
}
template <class Site> table<float, device_> trapz(const table<float, Site> &t)
{
    return trapz(t, detail::first_non_singleton(t.extent()));
}

template <class Site> table<float, device_> median(const table<float, Site> &t, int dim)
{
    return detail::median_dim(t, dim, NT2G_MEDIAN);
}
template <class Site> table<float, device_> median(const table<float, Site> &t)
{
    return detail::median_dim(t, detail::first_non_singleton(t.extent()), NT2G_MEDIAN);
}
template <class Site> table<float, device_> medianad(const table<float, Site> &t, int dim)
{
    return detail::median_dim(t, dim, NT2G_MEDIANAD);
}
template <class Site> table<float, device_> medianad(const table<float, Site> &t)
{
    return detail::median_dim(t, detail::first_non_singleton(t.extent()), NT2G_MEDIANAD);
}
template <class Site> float globalmedian(const table<float, Site> &t) { return detail::median_all(t, NT2G_MEDIAN); }
template <class Site> float globalmedianad(const table<float, Site> &t)
{
    return detail::median_all(t, NT2G_MEDIANAD);
}

template <class Site> table<float, Site> cumsum(const table<float, Site> &t, int dim) { return detail::scan_dim(t, dim, NT2G_SCAN_SUM); }
template <class Site> table<float, Site> cumprod(const table<float, Site> &t, int dim) { return detail::scan_dim(t, dim, NT2G_SCAN_PROD); }
template <class Site> table<float, Site> cummax(const table<float, Site> &t, int dim) { return detail::scan_dim(t, dim, NT2G_SCAN_MAX); }
template <class Site> table<float, Site> cummin(const table<float, Site> &t, int dim) { return detail::scan_dim(t, dim, NT2G_SCAN_MIN); }
// cumsum(t): along the first non-singleton dimension
template <class Site> table<float, Site> cumsum(const table<float, Site> &t)
{
    return detail::scan_dim(t, detail::first_non_singleton(t.extent()), NT2G_SCAN_SUM);
}

// sum(a) of a table with more than one non-singleton dimension folds the first of them
template <class Site> table<float, Site> sum_first(const table<float, Site> &t)
{
    return detail::fold_dim(t, detail::first_non_singleton(t.extent()), NT2G_FOLD_SUM);
}

}  // namespace nt2
