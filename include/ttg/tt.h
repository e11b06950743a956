// Edges, terminals, template tasks (TTs), make_tt, send/broadcast and graph utilities of the TTG
// API (ttg/ttg/edge.h, terminal.h, tt.h, make_tt.h:488-598, func.h:78-330) on the GB300 runtime.
//
// A TT keeps a table of pending task instances keyed by the task id; each input terminal fills
// one slot of the instance; when the last slot arrives the instance is queued with its priority
// (the semantics of the PaRSEC backend's set_arg_local_impl/release_task,
// ttg/ttg/parsec/ttg.h:2397-2727). Values travel as shared holders: consumers that take an input
// by const reference share one copy; a consumer that takes it by rvalue reference owns it — it is
// moved when it is the only consumer, deferred until the readers are done when the TT's
// defer_writer is set (parsec/ttg.h:4341), and deep-copied otherwise.
#pragma once
#include <algorithm>
#include <cassert>
#include <functional>
#include <iterator>
#include <map>
#include <memory>
#include <mutex>
#include <optional>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "ttg/buffer.h"
#include "ttg/runtime.h"

namespace ttg {

class TTBase;
class TerminalBase;
template <typename Key, typename Value>
class In;
template <typename Key, typename Value>
class Out;

namespace meta {
template <typename T>
inline constexpr bool is_void_v = std::is_void_v<T>;
template <typename T>
struct is_tuple : std::false_type {};
template <typename... Ts>
struct is_tuple<std::tuple<Ts...>> : std::true_type {};
template <typename T>
inline constexpr bool is_tuple_v = is_tuple<std::decay_t<T>>::value;
template <typename T, typename = void>
struct is_iterable : std::false_type {};
template <typename T>
struct is_iterable<T, std::void_t<decltype(std::begin(std::declval<T&>())), decltype(std::end(std::declval<T&>()))>>
    : std::true_type {};
template <typename T>
inline constexpr bool is_iterable_v = is_iterable<std::decay_t<T>>::value;
template <typename T>
inline constexpr bool is_const_v = std::is_const_v<std::remove_reference_t<T>>;
}  // namespace meta

// ---- shared value holders ----------------------------------------------------------------------
namespace detail {

struct HolderBase {
  virtual ~HolderBase() = default;
};

// One copy of a value in flight. `readers` counts const consumers not yet finished; a deferred
// writer is released when it drops to zero.
template <typename V>
struct Holder : HolderBase {
  V value;
  std::mutex m;
  int readers = 0;
  std::vector<std::function<void()>> deferred;
  explicit Holder(V&& v) : value(std::move(v)) {}
  explicit Holder(const V& v) : value(v) {}
  void reader_done() {
    std::vector<std::function<void()>> run;
    {
      std::lock_guard<std::mutex> lk(m);
      if (--readers == 0) run.swap(deferred);
    }
    for (auto& f : run) f();
  }
};

template <typename V>
using HolderPtr = std::shared_ptr<Holder<V>>;

template <typename V>
V deep_copy(V& v) {
  if constexpr (std::is_copy_constructible_v<V>) {
    sync_value_to_host(v);  // copy constructors read host data
    return V(static_cast<const V&>(v));
  } else {
    throw std::runtime_error("ttg: a move-only value cannot be given to more than one writer");
  }
}

// the running task's inputs: a value it sends on is forwarded (same holder), not copied — the
// reference's copy handler does the same for a task's own input data copies
struct InputRef {
  const void* addr;
  std::shared_ptr<HolderBase> holder;
};
inline std::vector<InputRef>*& tl_inputs() {
  thread_local std::vector<InputRef>* p = nullptr;
  return p;
}

// thread-local access to the running task's output terminals (implicit-terminal send<i>(...))
inline std::vector<TerminalBase*>*& tl_outputs() {
  thread_local std::vector<TerminalBase*>* p = nullptr;
  return p;
}

// One receiver of a value: an input terminal and the key it gets the value under.
struct Consumer {
  bool is_const;
  bool defer;
  std::function<void(std::shared_ptr<HolderBase>, bool owned)> deliver;
};

// The sharing policy for one value sent to a set of consumers (one send or one broadcast across
// terminals): const consumers share a single holder; the first mutable consumer owns it — at once
// when there are no readers, after the readers when it defers writes — and every other mutable
// consumer gets a deep copy taken before anyone runs.
template <typename D>
void dispatch_value(std::vector<Consumer>& cons, std::pair<std::shared_ptr<Holder<D>>, bool> hp) {
  auto& h = hp.first;
  const bool forwarded = hp.second;  // an input of the sending task: it may still be reading it
  if (cons.empty()) return;
  if (cons.size() == 1 && !forwarded) {
    cons[0].deliver(std::move(h), true);
    return;
  }
  int nreaders = 0;
  for (auto& c : cons) nreaders += c.is_const ? 1 : 0;
  int readers_now;
  {
    std::lock_guard<std::mutex> lk(h->m);
    h->readers += nreaders;
    readers_now = h->readers;
  }
  bool owner_given = false;
  for (auto& c : cons) {
    if (c.is_const) continue;
    if (!owner_given && (readers_now == 0 || c.defer)) {
      owner_given = true;
      if (readers_now == 0) {
        c.deliver(h, true);
      } else {
        std::lock_guard<std::mutex> lk(h->m);
        h->deferred.push_back([d = c.deliver, h]() { d(h, true); });
      }
    } else {
      c.deliver(std::make_shared<Holder<D>>(deep_copy(h->value)), true);
    }
  }
  for (auto& c : cons)
    if (c.is_const) c.deliver(h, false);
}

template <typename D, typename V>
std::pair<std::shared_ptr<Holder<D>>, bool> make_holder(V&& value) {
  if constexpr (std::is_lvalue_reference_v<V>) {
    if (auto* ins = tl_inputs()) {
      for (auto& r : *ins)
        if (r.addr == static_cast<const void*>(&value)) {
          if (auto hh = std::dynamic_pointer_cast<Holder<D>>(r.holder)) return {hh, true};
        }
    }
    D copy = deep_copy(const_cast<D&>(static_cast<const D&>(value)));
    return {std::make_shared<Holder<D>>(std::move(copy)), false};
  } else {
    return {std::make_shared<Holder<D>>(std::move(value)), false};
  }
}
}  // namespace detail

// ---- terminals -----------------------------------------------------------------------------------
class TerminalBase {
 public:
  enum class Type { Write, Read, Consume };
  virtual ~TerminalBase() = default;
  TTBase* get_tt() const { return tt_; }
  size_t get_index() const { return index_; }
  const std::string& get_name() const { return name_; }
  void set(TTBase* tt, size_t index, const std::string& name) {
    tt_ = tt;
    index_ = index;
    name_ = name;
  }
  const std::vector<TerminalBase*>& get_connections() const { return successors_; }
  const std::vector<TerminalBase*>& get_predecessors() const { return predecessors_; }
  void add_predecessor(TerminalBase* p) { predecessors_.push_back(p); }
  virtual bool is_input() const = 0;
  bool is_connected() const { return connected_; }

 protected:
  TTBase* tt_ = nullptr;
  size_t index_ = 0;
  std::string name_;
  std::vector<TerminalBase*> successors_, predecessors_;
  bool connected_ = false;
  friend class TTBase;
};

/// Input terminal: delivers (key, value holder) into its TT's task table.
template <typename Key, typename Value>
class In : public TerminalBase {
 public:
  using key_type = Key;
  using value_type = Value;
  // how the owning TT consumes this input: const (shared read) or mutable (owned)
  bool is_const_input = true;
  bool defer_writer = false;
  std::function<void(const Key*, std::shared_ptr<detail::HolderBase>, bool owned)> deliver;
  bool is_input() const override { return true; }
  void mark_connected() { connected_ = true; }
};

/// Output terminal: sends keys/values to every connected input terminal.
template <typename Key, typename Value>
class Out : public TerminalBase {
 public:
  using key_type = Key;
  using value_type = Value;
  bool is_input() const override { return false; }

  void connect(In<Key, Value>* in) {
    if (std::find(ins_.begin(), ins_.end(), in) != ins_.end()) return;
    ins_.push_back(in);
    successors_.push_back(in);
    connected_ = true;
    in->mark_connected();
    in->add_predecessor(this);
  }
  size_t nsuccessors() const { return ins_.size(); }

  // ---- valued sends
  template <typename K = Key, typename V>
  std::enable_if_t<!std::is_void_v<K> && !std::is_void_v<Value>> send(const K& key, V&& value) {
    std::vector<detail::Consumer> cons;
    collect(Key(key), cons);
    detail::dispatch_value<std::decay_t<Value>>(cons, detail::make_holder<std::decay_t<Value>>(std::forward<V>(value)));
  }
  template <typename Range, typename V>
  std::enable_if_t<!std::is_void_v<Value> && meta::is_iterable_v<Range>> broadcast(const Range& keylist, V&& value) {
    std::vector<detail::Consumer> cons;
    for (const auto& k : keylist) collect(Key(k), cons);
    detail::dispatch_value<std::decay_t<Value>>(cons, detail::make_holder<std::decay_t<Value>>(std::forward<V>(value)));
  }
  template <typename V, typename VV = Value>
  std::enable_if_t<!std::is_void_v<VV>> sendv(V&& value) {
    static_assert(std::is_void_v<Key>, "sendv needs a void key");
    std::vector<detail::Consumer> cons;
    collect_void(cons);
    detail::dispatch_value<std::decay_t<Value>>(cons, detail::make_holder<std::decay_t<Value>>(std::forward<V>(value)));
  }
  // ---- control-only sends
  template <typename K = Key>
  std::enable_if_t<!std::is_void_v<K> && std::is_void_v<Value>> sendk(const K& key) {
    const Key k(key);
    for (auto* in : ins_) in->deliver(&k, nullptr, true);
  }
  template <typename K = Key>
  std::enable_if_t<std::is_void_v<K> && std::is_void_v<Value>> send() {
    for (auto* in : ins_) in->deliver(nullptr, nullptr, true);
  }
  template <typename Range>
  std::enable_if_t<std::is_void_v<Value> && meta::is_iterable_v<Range>> broadcast(const Range& keylist) {
    for (const auto& k : keylist) sendk(Key(k));
  }
  template <typename K = Key>
  std::enable_if_t<!std::is_void_v<K> && std::is_void_v<Value>> send(const K& key) {
    sendk(key);
  }
  // device-send hook of the reference (terminal.h prepare_send): coherence is handled at delivery
  template <typename... Args>
  void prepare_send(Args&&...) {}

  /// Appends this terminal's receivers of `key` (used by multi-terminal broadcasts).
  template <typename K = Key>
  void collect(const K& key, std::vector<detail::Consumer>& cons) {
    for (auto* in : ins_) {
      Key k(key);
      cons.push_back(detail::Consumer{in->is_const_input, in->defer_writer,
                                      [in, k](std::shared_ptr<detail::HolderBase> h, bool owned) {
                                        in->deliver(&k, std::move(h), owned);
                                      }});
    }
  }
  void collect_void(std::vector<detail::Consumer>& cons) {
    for (auto* in : ins_)
      cons.push_back(detail::Consumer{in->is_const_input, in->defer_writer,
                                      [in](std::shared_ptr<detail::HolderBase> h, bool owned) {
                                        in->deliver(nullptr, std::move(h), owned);
                                      }});
  }

 private:
  std::vector<In<Key, Value>*> ins_;
};

// ---- edges ---------------------------------------------------------------------------------------
template <typename Key = void, typename Value = void>
class Edge {
  struct Impl {
    std::string name;
    std::vector<Out<Key, Value>*> outs;
    std::vector<In<Key, Value>*> ins;
  };
  std::vector<std::shared_ptr<Impl>> impls_;

 public:
  using key_type = Key;
  using value_type = Value;
  using output_terminal_type = Out<Key, Value>;
  explicit Edge(const std::string& name = "anonymous edge") : impls_{std::make_shared<Impl>()} {
    impls_[0]->name = name;
  }
  template <typename... Es>
  explicit Edge(const Edge& e, const Es&... es) {  // fuse
    impls_ = e.impls_;
    (impls_.insert(impls_.end(), es.impls_.begin(), es.impls_.end()), ...);
  }
  const std::string& get_name() const { return impls_[0]->name; }
  void set_in(In<Key, Value>* in) const {
    for (auto& p : impls_) {
      p->ins.push_back(in);
      for (auto* o : p->outs) o->connect(in);
    }
  }
  void set_out(Out<Key, Value>* out) const {
    for (auto& p : impls_) {
      p->outs.push_back(out);
      for (auto* i : p->ins) out->connect(i);
    }
  }
  template <typename K, typename V>
  friend class Edge;
};

template <typename... Es>
auto edges(Es&&... es) {
  return std::make_tuple(std::forward<Es>(es)...);
}
template <typename Key, typename Value, typename... Es>
Edge<Key, Value> fuse(const Edge<Key, Value>& e, const Es&... es) {
  return Edge<Key, Value>(e, es...);
}

template <typename T>
struct edges_to_output_terminals;
template <typename... Es>
struct edges_to_output_terminals<std::tuple<Es...>> {
  using type = std::tuple<typename std::decay_t<Es>::output_terminal_type...>;
};

// ---- TT base ---------------------------------------------------------------------------------------
class TTBase {
 public:
  virtual ~TTBase() = default;
  const std::string& get_name() const { return name_; }
  void set_name(const std::string& n) { name_ = n; }
  virtual std::vector<TerminalBase*> get_inputs_base() { return ins_base_; }
  virtual std::vector<TerminalBase*> get_outputs_base() { return outs_base_; }
  TerminalBase* in(size_t i) { return ins_base_.at(i); }
  TerminalBase* out(size_t i) { return outs_base_.at(i); }
  bool is_executable() const { return executable_; }
  virtual void make_executable() { executable_ = true; }
  virtual bool is_composite() const { return false; }
  virtual std::vector<TTBase*> get_ops() { return {}; }
  void set_trace_instance(bool) {}
  size_t num_tasks_pending() const { return pending_count_; }

 protected:
  std::string name_;
  std::vector<TerminalBase*> ins_base_, outs_base_;
  bool executable_ = false;
  size_t pending_count_ = 0;
};

template <typename Key>
using keymap_fn_t = std::function<int(const Key&)>;

namespace detail {
// Argument binding: for each input value type decide whether func takes it mutable (V&&) or
// read-only (const V&). Non-generic callables are read from their signature; generic ones take
// an input read-only only if they cannot accept it as an rvalue.
template <typename F>
struct callable_args {
  static constexpr bool generic = true;
};
template <typename F, typename = void>
struct is_generic : std::true_type {};
template <typename F>
struct is_generic<F, std::void_t<decltype(&std::decay_t<F>::operator())>> : std::false_type {};

template <typename T>
struct memfn_args;
template <typename C, typename R, typename... A>
struct memfn_args<R (C::*)(A...) const> {
  using type = std::tuple<A...>;
  using ret = R;
};
template <typename C, typename R, typename... A>
struct memfn_args<R (C::*)(A...)> {
  using type = std::tuple<A...>;
  using ret = R;
};
template <typename C, typename R, typename... A>
struct memfn_args<R (C::*)(A...) const noexcept> {
  using type = std::tuple<A...>;
  using ret = R;
};
template <typename C, typename R, typename... A>
struct memfn_args<R (C::*)(A...) noexcept> {
  using type = std::tuple<A...>;
  using ret = R;
};

template <typename A>
inline constexpr bool arg_is_mutable =
    std::is_rvalue_reference_v<A> || (!std::is_reference_v<A> && !std::is_const_v<A>);

template <typename T>
struct type_tag {
  using type = T;
};
}  // namespace detail

// ---- input mutability from the callable's signature ---------------------------------------------
namespace detail {
template <typename T>
struct always_false : std::false_type {};

// index of the function argument that receives input I (void inputs have none)
template <bool VoidKey, typename... Values>
constexpr std::array<int, sizeof...(Values) + 1> input_arg_positions() {
  std::array<int, sizeof...(Values) + 1> pos{};
  constexpr bool isvoid[] = {std::is_void_v<Values>..., false};
  int a = VoidKey ? 0 : 1;
  for (size_t i = 0; i + 1 < sizeof...(Values) + 1; ++i) pos[i] = isvoid[i] ? -1 : a++;
  return pos;
}

template <typename Args, int Pos>
constexpr bool arg_mutable_at() {
  if constexpr (Pos < 0) return true;
  else if constexpr ((size_t)Pos < std::tuple_size_v<Args>) return arg_is_mutable<std::tuple_element_t<(size_t)Pos, Args>>;
  else return true;
}

template <typename Func, bool VoidKey, typename... Values, size_t... I>
constexpr std::array<bool, sizeof...(Values) + 1> input_mutability_impl(std::index_sequence<I...>) {
  using args = typename memfn_args<decltype(&std::decay_t<Func>::operator())>::type;
  constexpr auto pos = input_arg_positions<VoidKey, Values...>();
  return std::array<bool, sizeof...(Values) + 1>{arg_mutable_at<args, pos[I]>()..., true};
}

template <typename Func, bool VoidKey, typename... Values>
constexpr std::array<bool, sizeof...(Values) + 1> input_mutability() {
  if constexpr (!is_generic<Func>::value) {
    return input_mutability_impl<Func, VoidKey, Values...>(std::make_index_sequence<sizeof...(Values)>{});
  } else {
    std::array<bool, sizeof...(Values) + 1> mut{};
    for (size_t i = 0; i < sizeof...(Values) + 1; ++i) mut[i] = true;  // generic: bind inputs as rvalues
    return mut;
  }
}
}  // namespace detail

// ---- the template task -----------------------------------------------------------------------------
template <ExecutionSpace Space, typename Key, typename Func, typename OutTerms, typename... Values>
class TT : public TTBase {
  static constexpr size_t numins = sizeof...(Values);
  static constexpr bool void_key = std::is_void_v<Key>;

 public:
  using key_store = std::conditional_t<void_key, int, Key>;

 private:
  template <size_t I>
  using value_t = std::tuple_element_t<I, std::tuple<Values...>>;
  static constexpr auto kMut = detail::input_mutability<Func, void_key, Values...>();

  struct Pending {
    std::array<std::shared_ptr<detail::HolderBase>, numins == 0 ? 1 : numins> h;
    std::array<bool, numins == 0 ? 1 : numins> owned{};
    std::array<bool, numins == 0 ? 1 : numins> have{};
    int count = 0;
  };

  Func func_;
  std::tuple<In<Key, Values>...> ins_;
  OutTerms outs_;
  std::vector<TerminalBase*> out_ptrs_;
  std::mutex m_;
  std::unordered_map<key_store, Pending> table_;
  std::function<int64_t(const key_store&)> priomap_;
  std::function<int(const key_store&)> devicemap_;
  std::function<int(const key_store&)> keymap_;
  bool defer_writer_ = false;

 public:
  using key_type = Key;
  using input_values_tuple_type = std::tuple<Values...>;
  using output_terminals_type = OutTerms;
  static constexpr ExecutionSpace space = Space;

  template <typename InEdges, typename OutEdges>
  TT(Func&& f, const InEdges& inedges, const OutEdges& outedges, const std::string& name,
     const std::vector<std::string>& innames, const std::vector<std::string>& outnames)
      : func_(std::move(f)) {
    name_ = name;
    init_inputs(inedges, innames, std::make_index_sequence<numins>{});
    init_outputs(outedges, outnames, std::make_index_sequence<std::tuple_size_v<OutTerms>>{});
  }
  TT(const TT&) = delete;

  template <size_t i>
  auto* in() {
    return &std::get<i>(ins_);
  }
  template <size_t i>
  auto* out() {
    return &std::get<i>(outs_);
  }
  OutTerms& get_output_terminals() { return outs_; }

  template <typename F>
  void set_keymap(F&& f) {
    if constexpr (void_key) keymap_ = [g = std::forward<F>(f)](const int&) { return (int)g(); };
    else keymap_ = [g = std::forward<F>(f)](const Key& k) { return (int)g(k); };
  }
  template <typename F>
  void set_priomap(F&& f) {
    if constexpr (void_key) priomap_ = [g = std::forward<F>(f)](const int&) { return (int64_t)g(); };
    else priomap_ = [g = std::forward<F>(f)](const Key& k) { return (int64_t)g(k); };
  }
  template <typename F>
  void set_devicemap(F&& f) {
    if constexpr (void_key) devicemap_ = [g = std::forward<F>(f)](const int&) { return (int)g(); };
    else devicemap_ = [g = std::forward<F>(f)](const Key& k) { return (int)g(k); };
  }
  void set_defer_writer(bool v) {
    defer_writer_ = v;
    set_defer_all(std::make_index_sequence<numins>{});
  }
  bool get_defer_writer() const { return defer_writer_; }

  /// Starts one task instance with all inputs given (the TT::invoke of parsec/ttg.h:4238-4340).
  template <typename K = Key, typename... Args>
  std::enable_if_t<!std::is_void_v<K>> invoke(const K& key, Args&&... args) {
    invoke_impl(&key, std::forward<Args>(args)...);
  }
  template <typename K = Key, typename... Args>
  std::enable_if_t<std::is_void_v<K>> invoke(Args&&... args) {
    invoke_impl(nullptr, std::forward<Args>(args)...);
  }

  void make_executable() override { executable_ = true; }

 private:
  template <typename... Args>
  void invoke_impl(const void* keyp, Args&&... args) {
    if constexpr (numins == 0) {
      static_assert(sizeof...(Args) == 0, "this TT has no inputs");
      key_store k{};
      if constexpr (!void_key) k = *static_cast<const Key*>(keyp);
      schedule(k, Pending{});
    } else if constexpr (sizeof...(Args) == 0) {
      invoke_void_inputs(keyp, std::make_index_sequence<numins>{});
    } else {
      static_assert(sizeof...(Args) == numins, "invoke needs a value for every input");
      invoke_values(keyp, std::make_index_sequence<numins>{}, std::forward<Args>(args)...);
    }
  }
  template <size_t... I>
  void invoke_void_inputs(const void* keyp, std::index_sequence<I...>) {
    (set_arg<I>(static_cast<const Key*>(keyp), nullptr, true), ...);
  }
  template <size_t... I, typename... Args>
  void invoke_values(const void* keyp, std::index_sequence<I...>, Args&&... args) {
    (set_arg<I>(static_cast<const Key*>(keyp), make_value_holder<value_t<I>>(std::forward<Args>(args)), true), ...);
  }
  template <typename V, typename A>
  static std::shared_ptr<detail::HolderBase> make_value_holder(A&& a) {
    using D = std::decay_t<V>;
    if constexpr (std::is_void_v<V>) return nullptr;
    else if constexpr (std::is_lvalue_reference_v<A>)
      return std::make_shared<detail::Holder<D>>(detail::deep_copy(const_cast<D&>(static_cast<const D&>(a))));
    else
      return std::make_shared<detail::Holder<D>>(D(std::move(a)));
  }

  template <typename InEdges, size_t... I>
  void init_inputs(const InEdges& inedges, const std::vector<std::string>& names, std::index_sequence<I...>) {
    (init_input<I>(std::get<I>(inedges), I < names.size() ? names[I] : std::string("input")), ...);
  }
  template <size_t I, typename E>
  void init_input(const E& e, const std::string& nm) {
    auto& t = std::get<I>(ins_);
    t.set(this, I, nm);
    t.is_const_input = !kMut[I];
    t.deliver = [this](const Key* k, std::shared_ptr<detail::HolderBase> h, bool owned) {
      set_arg<I>(k, std::move(h), owned);
    };
    ins_base_.push_back(&t);
    e.set_in(&t);
  }
  template <typename OutEdges, size_t... I>
  void init_outputs(const OutEdges& outedges, const std::vector<std::string>& names, std::index_sequence<I...>) {
    (init_output<I>(std::get<I>(outedges), I < names.size() ? names[I] : std::string("output")), ...);
  }
  template <size_t I, typename E>
  void init_output(const E& e, const std::string& nm) {
    auto& t = std::get<I>(outs_);
    t.set(this, I, nm);
    outs_base_.push_back(&t);
    out_ptrs_.push_back(&t);
    e.set_out(&t);
  }
  template <size_t... I>
  void set_defer_all(std::index_sequence<I...>) {
    ((std::get<I>(ins_).defer_writer = defer_writer_), ...);
  }

  template <size_t I>
  void set_arg(const Key* kp, std::shared_ptr<detail::HolderBase> h, bool owned) {
    key_store k{};
    if constexpr (!void_key) k = *kp;
    Pending ready;
    bool fire = false;
    {
      std::lock_guard<std::mutex> lk(m_);
      auto& p = table_[k];
      if (p.have[I]) {
        std::ostringstream os;
        os << "ttg: input " << I << " of " << name_ << " received twice for key ";
        if constexpr (!void_key) os << k;
        throw std::runtime_error(os.str());
      }
      p.have[I] = true;
      p.h[I] = std::move(h);
      p.owned[I] = owned;
      if (++p.count == (int)numins) {
        ready = std::move(p);
        table_.erase(k);
        fire = true;
      }
      pending_count_ = table_.size();
    }
    if (fire) schedule(k, std::move(ready));
  }

  int64_t priority(const key_store& k) const { return priomap_ ? priomap_(k) : 0; }

  void schedule(const key_store& k, Pending&& p) {
    auto sp = std::make_shared<Pending>(std::move(p));
    rt::Runtime::get().submit(priority(k), [this, k, sp]() { run_task(k, sp); });
  }

  // release the holders of a finished task (const readers let deferred writers go)
  void release_inputs(Pending& p) { release_impl(p, std::make_index_sequence<numins>{}); }
  template <size_t... I>
  void release_impl(Pending& p, std::index_sequence<I...>) {
    (release_one<I>(p), ...);
  }
  template <size_t I>
  void release_one(Pending& p) {
    if constexpr (!std::is_void_v<value_t<I>>) {
      if (p.h[I] && !p.owned[I]) static_cast<detail::Holder<std::decay_t<value_t<I>>>*>(p.h[I].get())->reader_done();
    }
    p.h[I].reset();
  }

  template <size_t... I>
  void sync_inputs_to_host(Pending& p, std::index_sequence<I...>) {
    (sync_one<I>(p), ...);
  }
  template <size_t... I>
  bool inputs_on_device(Pending& p, std::index_sequence<I...>) {
    return (on_device_one<I>(p) || ... || false);
  }
  template <size_t I>
  bool on_device_one(Pending& p) {
    if constexpr (!std::is_void_v<value_t<I>>) {
      using V = std::decay_t<value_t<I>>;
      return detail::value_on_device(static_cast<detail::Holder<V>*>(p.h[I].get())->value);
    } else {
      return false;
    }
  }
  template <size_t I>
  void sync_one(Pending& p) {
    if constexpr (!std::is_void_v<value_t<I>>) {
      using V = std::decay_t<value_t<I>>;
      detail::sync_value_to_host(static_cast<detail::Holder<V>*>(p.h[I].get())->value);
    }
  }

  // the reference-typed argument of input I: () for void, (const V&) or (V&&)
  template <size_t I>
  auto arg_tuple(Pending& p) {
    if constexpr (std::is_void_v<value_t<I>>) {
      return std::tuple<>{};
    } else {
      using V = std::decay_t<value_t<I>>;
      auto* holder = static_cast<detail::Holder<V>*>(p.h[I].get());
      if constexpr (kMut[I]) return std::tuple<V&&>(std::move(holder->value));
      else return std::tuple<const V&>(holder->value);
    }
  }
  template <size_t... I>
  void input_refs(Pending& p, std::vector<detail::InputRef>& v, std::index_sequence<I...>) {
    (input_ref<I>(p, v), ...);
  }
  template <size_t I>
  void input_ref(Pending& p, std::vector<detail::InputRef>& v) {
    if constexpr (!std::is_void_v<value_t<I>>) {
      using V = std::decay_t<value_t<I>>;
      if (p.h[I]) v.push_back({&static_cast<detail::Holder<V>*>(p.h[I].get())->value, p.h[I]});
    }
  }
  template <size_t... I>
  auto all_args(Pending& p, std::index_sequence<I...>) {
    return std::tuple_cat(arg_tuple<I>(p)...);
  }
  template <typename... A>
  decltype(auto) call_with(const key_store& k, A&&... a) {
    if constexpr (void_key) {
      if constexpr (std::is_invocable_v<Func&, A&&..., OutTerms&>) return func_(std::forward<A>(a)..., outs_);
      else return func_(std::forward<A>(a)...);
    } else {
      if constexpr (std::is_invocable_v<Func&, const Key&, A&&..., OutTerms&>)
        return func_(static_cast<const Key&>(k), std::forward<A>(a)..., outs_);
      else return func_(static_cast<const Key&>(k), std::forward<A>(a)...);
    }
  }
  decltype(auto) call_body(const key_store& k, Pending& p) {
    return std::apply([&](auto&&... a) -> decltype(auto) { return call_with(k, std::forward<decltype(a)>(a)...); },
                      all_args(p, std::make_index_sequence<numins>{}));
  }

  void run_task(const key_store& k, std::shared_ptr<Pending> sp);
  int stream_hint(const key_store& k) const { return devicemap_ ? -1 : -1; }

  template <typename T>
  friend struct DeviceDriver;
};

// ---- make_tt (ttg/ttg/make_tt.h:488-578) ----------------------------------------------------------
namespace detail {
template <typename Key, typename InEdges>
struct edges_key;
template <typename Key>
struct edges_key<Key, std::tuple<>> {
  using type = Key;
};
template <typename Key, typename K0, typename V0, typename... R>
struct edges_key<Key, std::tuple<Edge<K0, V0>, R...>> {
  using type = std::conditional_t<std::is_void_v<Key>, K0, Key>;
};
}  // namespace detail

template <ExecutionSpace Space, typename keyT = void, typename funcT, typename... input_edge_valuesT,
          typename... output_edgesT>
auto make_tt(funcT&& func, const std::tuple<Edge<keyT, input_edge_valuesT>...>& inedges = std::tuple<>{},
             const std::tuple<output_edgesT...>& outedges = std::tuple<>{}, const std::string& name = "wrapper",
             const std::vector<std::string>& innames = std::vector<std::string>(sizeof...(input_edge_valuesT), "input"),
             const std::vector<std::string>& outnames = std::vector<std::string>(sizeof...(output_edgesT), "output")) {
  using OutTerms = typename edges_to_output_terminals<std::tuple<output_edgesT...>>::type;
  using F = std::decay_t<funcT>;
  using TTT = TT<Space, keyT, F, OutTerms, input_edge_valuesT...>;
  return std::make_unique<TTT>(F(std::forward<funcT>(func)), inedges, outedges, name, innames, outnames);
}

// keys of input edges deduce keyT (an explicit first argument fixes it, e.g. make_tt<void>(...) for
// a task without a key)
template <typename keyT = void, typename funcT, typename... input_edge_valuesT, typename... output_edgesT>
auto make_tt(funcT&& func, const std::tuple<Edge<keyT, input_edge_valuesT>...>& inedges = std::tuple<>{},
             const std::tuple<output_edgesT...>& outedges = std::tuple<>{}, const std::string& name = "wrapper",
             const std::vector<std::string>& innames = std::vector<std::string>(sizeof...(input_edge_valuesT), "input"),
             const std::vector<std::string>& outnames = std::vector<std::string>(sizeof...(output_edgesT), "output")) {
  return make_tt<ExecutionSpace::Host, keyT>(std::forward<funcT>(func), inedges, outedges, name, innames, outnames);
}

// ---- send / broadcast with explicit or implicit terminals (ttg/ttg/func.h:157-330) ---------------
namespace detail {
template <typename Key, typename Value>
Out<Key, Value>* get_out_terminal(size_t i, const char* what) {
  auto* outs = tl_outputs();
  if (!outs || i >= outs->size()) throw std::runtime_error(std::string(what) + ": no such output terminal");
  auto* t = dynamic_cast<Out<Key, std::decay_t<Value>>*>((*outs)[i]);
  if (!t) throw std::runtime_error(std::string(what) + ": output terminal type mismatch");
  return t;
}
}  // namespace detail

template <size_t i, typename keyT, typename valueT, typename... out_keysT, typename... out_valuesT>
inline void send(const keyT& key, valueT&& value, std::tuple<Out<out_keysT, out_valuesT>...>& t) {
  std::get<i>(t).send(key, std::forward<valueT>(value));
}
template <size_t i, typename keyT, typename valueT>
inline void send(const keyT& key, valueT&& value) {
  using OK = std::decay_t<keyT>;
  detail::get_out_terminal<OK, std::decay_t<valueT>>(i, "ttg::send")->send(key, std::forward<valueT>(value));
}
template <size_t i, typename keyT, typename... out_keysT, typename... out_valuesT>
inline void sendk(const keyT& key, std::tuple<Out<out_keysT, out_valuesT>...>& t) {
  std::get<i>(t).sendk(key);
}
template <size_t i, typename keyT>
inline void sendk(const keyT& key) {
  detail::get_out_terminal<std::decay_t<keyT>, void>(i, "ttg::sendk")->sendk(key);
}
template <size_t i, typename valueT, typename... out_keysT, typename... out_valuesT>
inline void sendv(valueT&& value, std::tuple<Out<out_keysT, out_valuesT>...>& t) {
  std::get<i>(t).sendv(std::forward<valueT>(value));
}
template <size_t i, typename... out_keysT, typename... out_valuesT>
inline void send(std::tuple<Out<out_keysT, out_valuesT>...>& t) {
  std::get<i>(t).send();
}


namespace detail {
template <size_t KeyId, size_t I, size_t... Is, typename KL, typename Outs>
void collect_multi(const KL& keylists, Outs& t, std::vector<Consumer>& cons) {
  const auto& kl = std::get<KeyId>(keylists);
  auto& term = std::get<I>(t);
  using TK = typename std::decay_t<decltype(term)>::key_type;
  if constexpr (meta::is_iterable_v<std::decay_t<decltype(kl)>> && !std::is_same_v<std::decay_t<decltype(kl)>, TK>) {
    for (const auto& k : kl) term.collect(TK(k), cons);
  } else {
    term.collect(TK(kl), cons);
  }
  if constexpr (sizeof...(Is) > 0) collect_multi<KeyId + 1, Is...>(keylists, t, cons);
}
template <size_t I, size_t... Is, typename KL, typename valueT, typename Outs>
void broadcast_multi(const KL& keylists, valueT&& value, Outs& t) {
  using D = typename std::decay_t<std::tuple_element_t<I, Outs>>::value_type;
  std::vector<Consumer> cons;
  collect_multi<0, I, Is...>(keylists, t, cons);
  dispatch_value<std::decay_t<D>>(cons, make_holder<std::decay_t<D>>(std::forward<valueT>(value)));
}
}  // namespace detail

/// broadcast<I, Is...>(keylists, value, out): every terminal I, Is... gets the value for each key
/// of its keylist (a single key or a range). All sends share one value copy.
template <size_t I, size_t... Is, typename rangeT, typename valueT, typename... out_keysT, typename... out_valuesT>
inline void broadcast(const rangeT& keylists, valueT&& value, std::tuple<Out<out_keysT, out_valuesT>...>& t) {
  if constexpr (meta::is_tuple_v<rangeT>) {
    static_assert(sizeof...(Is) + 1 == std::tuple_size_v<std::decay_t<rangeT>>, "one keylist per terminal");
    detail::broadcast_multi<I, Is...>(keylists, std::forward<valueT>(value), t);
  } else {
    detail::broadcast_multi<I>(std::tie(keylists), std::forward<valueT>(value), t);
  }
}
template <size_t I, size_t... Is, typename rangeT, typename... out_keysT, typename... out_valuesT>
inline void broadcastk(const rangeT& keylists, std::tuple<Out<out_keysT, out_valuesT>...>& t) {
  if constexpr (meta::is_tuple_v<rangeT>) {
    [&]<size_t... J>(std::index_sequence<J...>) {
      constexpr size_t terms[] = {I, Is...};
      (std::get<terms[J]>(t).broadcast(std::get<J>(keylists)), ...);
    }(std::make_index_sequence<sizeof...(Is) + 1>{});
  } else {
    std::get<I>(t).broadcast(keylists);
  }
}

// ---- composites, traversal, executable graphs ----------------------------------------------------
template <typename InsTuple, typename OutsTuple>
class TTG : public TTBase {
  std::vector<std::unique_ptr<TTBase>> ops_;
  InsTuple ins_;
  OutsTuple outs_;

 public:
  TTG(std::vector<std::unique_ptr<TTBase>>&& ops, InsTuple ins, OutsTuple outs, const std::string& name)
      : ops_(std::move(ops)), ins_(ins), outs_(outs) {
    name_ = name;
    std::apply([&](auto*... p) { (ins_base_.push_back(p), ...); }, ins_);
    std::apply([&](auto*... p) { (outs_base_.push_back(p), ...); }, outs_);
  }
  template <size_t i>
  auto* in() {
    return std::get<i>(ins_);
  }
  template <size_t i>
  auto* out() {
    return std::get<i>(outs_);
  }
  bool is_composite() const override { return true; }
  std::vector<TTBase*> get_ops() override {
    std::vector<TTBase*> v;
    for (auto& p : ops_) v.push_back(p.get());
    return v;
  }
  void make_executable() override {
    for (auto& p : ops_) p->make_executable();
    executable_ = true;
  }
};

template <typename InsTuple, typename OutsTuple>
auto make_ttg(std::vector<std::unique_ptr<TTBase>>&& ops, const InsTuple& ins, const OutsTuple& outs,
              const std::string& name = "ttg") {
  return std::make_unique<TTG<InsTuple, OutsTuple>>(std::move(ops), ins, outs, name);
}

namespace detail {
// every TT reachable through predecessors and successors (ttg/ttg/traverse.h:29-100)
inline void collect(TTBase* tt, std::set<TTBase*>& seen) {
  if (!tt || !seen.insert(tt).second) return;
  for (auto* o : tt->get_ops()) collect(o, seen);
  for (auto* in : tt->get_inputs_base())
    for (auto* pred : in->get_predecessors()) collect(pred->get_tt(), seen);
  for (auto* out : tt->get_outputs_base())
    for (auto* succ : out->get_connections()) collect(succ->get_tt(), seen);
}
}  // namespace detail

/// Makes every TT reachable from the given ones executable (ttg/ttg/func.h:78-87). Like the
/// reference's traversal it returns false, and names the terminal, when a reachable input or
/// output terminal is not connected.
template <typename... TTs>
bool make_graph_executable(TTs*... tts) {
  std::set<TTBase*> seen;
  (detail::collect(static_cast<TTBase*>(tts), seen), ...);
  bool connected = true;
  for (auto* t : seen) {
    t->make_executable();
    if (t->is_composite()) continue;
    int i = 0;
    for (auto* in : t->get_inputs_base()) {
      if (!in->is_connected()) {
        std::cout << "ttg::Traverse: " << t->get_name() << " input terminal #" << i << " " << in->get_name()
                  << " is not connected\n";
        connected = false;
      }
      ++i;
    }
    i = 0;
    for (auto* out : t->get_outputs_base()) {
      if (!out->is_connected()) {
        std::cout << "ttg::Traverse: " << t->get_name() << " output terminal #" << i << " " << out->get_name()
                  << " is not connected\n";
        connected = false;
      }
      ++i;
    }
  }
  return connected;
}
template <typename T>
bool make_graph_executable(const std::unique_ptr<T>& tt) {
  return make_graph_executable(tt.get());
}

/// DOT rendering of the graph reachable from a TT (ttg/ttg/util/dot.h).
class Dot {
 public:
  template <typename... TTs>
  std::string operator()(TTs*... tts) const {
    std::set<TTBase*> seen;
    (detail::collect(static_cast<TTBase*>(tts), seen), ...);
    std::ostringstream os;
    os << "digraph ttg {\n";
    for (auto* t : seen) {
      if (t->is_composite()) continue;
      os << "  n" << (const void*)t << " [label=\"" << t->get_name() << "\"];\n";
      for (auto* out : t->get_outputs_base())
        for (auto* succ : out->get_connections())
          os << "  n" << (const void*)t << " -> n" << (const void*)succ->get_tt() << " [label=\"" << out->get_name()
             << "\"];\n";
    }
    os << "}\n";
    return os.str();
  }
};

}  // namespace ttg
