// Minimal stand-in for hpx::program_options as used by the LULESH reference
// (lulesh.cc:2418-2432 registers the options, lulesh-util.cc:36-56 reads
// them). Test infrastructure only.
//
// Accepted command-line forms: "--name value", "--name=value" and bare
// switches "--name". HPX runtime options ("--hpx:threads=N") are consumed by
// hpx::init and not stored here.
#pragma once

#include <any>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace hpx {
namespace program_options {

class value_semantic {
   public:
    virtual ~value_semantic() = default;
    virtual std::any parse(const std::string& text) const = 0;
    virtual bool has_default() const = 0;
    virtual std::any default_any() const = 0;
};

template <class T>
class typed_value : public value_semantic {
   public:
    typed_value* default_value(const T& v) {
        def_ = v;
        has_def_ = true;
        return this;
    }
    std::any parse(const std::string& text) const override {
        std::istringstream in(text);
        T v{};
        in >> v;
        if (in.fail()) throw std::invalid_argument("bad option value: " + text);
        return std::any(v);
    }
    bool has_default() const override { return has_def_; }
    std::any default_any() const override { return std::any(def_); }

   private:
    T def_{};
    bool has_def_ = false;
};

template <>
inline std::any typed_value<std::string>::parse(const std::string& text) const {
    return std::any(text);
}

template <class T>
typed_value<T>* value() {
    return new typed_value<T>();
}

class variable_value {
   public:
    variable_value() = default;
    explicit variable_value(std::any v) : v_(std::move(v)) {}
    template <class T>
    const T& as() const {
        return *std::any_cast<T>(&v_);
    }
    bool empty() const { return !v_.has_value(); }

   private:
    std::any v_;
};

class variables_map {
   public:
    std::size_t count(const std::string& k) const { return m_.count(k); }
    const variable_value& operator[](const std::string& k) const {
        auto it = m_.find(k);
        if (it == m_.end()) throw std::out_of_range("option not set: " + k);
        return it->second;
    }
    void set(const std::string& k, std::any v) { m_[k] = variable_value(std::move(v)); }

   private:
    std::map<std::string, variable_value> m_;
};

class options_description {
   public:
    struct option {
        std::string name;
        std::shared_ptr<value_semantic> sem;  // null for a switch
    };

    class adder {
       public:
        explicit adder(options_description* d) : d_(d) {}
        adder& operator()(const char* name, const char* /*help*/) {
            d_->opts_.push_back(option{name, nullptr});
            return *this;
        }
        adder& operator()(const char* name, value_semantic* sem, const char* /*help*/) {
            d_->opts_.push_back(option{name, std::shared_ptr<value_semantic>(sem)});
            return *this;
        }

       private:
        options_description* d_;
    };

    adder add_options() { return adder(this); }

    const option* find(const std::string& name) const {
        for (const auto& o : opts_)
            if (o.name == name) return &o;
        return nullptr;
    }
    const std::vector<option>& all() const { return opts_; }

   private:
    std::vector<option> opts_;
};

}  // namespace program_options
}  // namespace hpx
