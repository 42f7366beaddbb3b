// ParameterObject.h — a minimal stand-in for the GenericParameters library (the
// reference fetches it at configure time, commit 42d52ad551fafba600ee99e59fb0f9c7b557e2ed,
// CMake/SetUpExternalProjects.cmake:31-38). Test infrastructure only: it lets the
// reference's own hot-path sources compile into the reference pin driver
// (oracle/build_ref_step.sh). It restates the library's published interface as the
// reference uses it: objects register named parameters bound to a member (or a getter
// and setter pair) and read or write them by id; labels, groups, descriptions, limits and
// visibility are accepted and not interpreted.
#pragma once
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace GenParam {

class ParameterBase {
 public:
  enum DataTypes {
    BOOL = 0, ENUM, STRING, VEC_FLOAT, VEC_DOUBLE, VEC_INT8, VEC_INT16, VEC_INT32, VEC_UINT8, VEC_UINT16,
    VEC_UINT32, FLOAT, DOUBLE, INT8, INT16, INT32, UINT8, UINT16, UINT32
  };
  template <typename T> using GetFunc = std::function<T()>;
  template <typename T> using SetFunc = std::function<void(T)>;
  template <typename T> using GetVecFunc = std::function<T *()>;
  template <typename T> using SetVecFunc = std::function<void(T *)>;

  ParameterBase(const std::string &name, const std::string &label, DataTypes type)
      : m_name(name), m_label(label), m_type(type) {}
  virtual ~ParameterBase() {}
  const std::string &getName() const { return m_name; }
  const std::string &getLabel() const { return m_label; }
  DataTypes getType() const { return m_type; }
  void setGroup(const std::string &g) { m_group = g; }
  const std::string &getGroup() const { return m_group; }
  void setDescription(const std::string &d) { m_description = d; }
  const std::string &getDescription() const { return m_description; }
  void setReadOnly(bool v) { m_readOnly = v; }
  bool getReadOnly() const { return m_readOnly; }
  void setVisible(bool v) { m_visible = v; }
  bool getVisible() const { return m_visible; }
  void setHotKey(const std::string &k) { m_hotKey = k; }

 protected:
  std::string m_name, m_label, m_group, m_description, m_hotKey;
  DataTypes m_type;
  bool m_readOnly = false, m_visible = true;
};

template <typename T>
class Parameter : public ParameterBase {
 public:
  Parameter(const std::string &name, const std::string &label, DataTypes type, T *p)
      : ParameterBase(name, label, type), m_get([p]() { return *p; }), m_set([p](T v) { *p = v; }) {}
  Parameter(const std::string &name, const std::string &label, DataTypes type, GetFunc<T> g, SetFunc<T> s)
      : ParameterBase(name, label, type), m_get(g), m_set(s) {}
  T getValue() const { return m_get(); }
  void setValue(T v) {
    if (m_set) m_set(v);
  }

 protected:
  GetFunc<T> m_get;
  SetFunc<T> m_set;
};

template <typename T>
class NumericParameter : public Parameter<T> {
 public:
  using Parameter<T>::Parameter;
  void setMinValue(T v) { m_min = v; }
  void setMaxValue(T v) { m_max = v; }
  T getMinValue() const { return m_min; }
  T getMaxValue() const { return m_max; }

 protected:
  T m_min{}, m_max{};
};

using FloatParameter = NumericParameter<float>;
using DoubleParameter = NumericParameter<double>;
using IntParameter = NumericParameter<int>;
using UnsignedIntParameter = NumericParameter<unsigned int>;
using BoolParameter = Parameter<bool>;
using StringParameter = Parameter<std::string>;

class EnumParameter : public Parameter<int> {
 public:
  using Parameter<int>::Parameter;
  void addEnumValue(const std::string &name, int &id) {
    id = (int)m_values.size();
    m_values.push_back(name);
  }
  const std::vector<std::string> &getEnumValues() const { return m_values; }

 protected:
  std::vector<std::string> m_values;
};

template <typename T>
class VectorParameter : public ParameterBase {
 public:
  VectorParameter(const std::string &name, const std::string &label, DataTypes type, unsigned int dim, T *p)
      : ParameterBase(name, label, type), m_dim(dim), m_get([p]() { return p; }),
        m_set([p, dim](T *v) { for (unsigned int k = 0; k < dim; k++) p[k] = v[k]; }) {}
  VectorParameter(const std::string &name, const std::string &label, DataTypes type, unsigned int dim,
                  GetVecFunc<T> g, SetVecFunc<T> s)
      : ParameterBase(name, label, type), m_dim(dim), m_get(g), m_set(s) {}
  unsigned int getDim() const { return m_dim; }
  T *getValue() const { return m_get(); }
  void setValue(T *v) {
    if (m_set) m_set(v);
  }

 protected:
  unsigned int m_dim;
  GetVecFunc<T> m_get;
  SetVecFunc<T> m_set;
};

using FloatVectorParameter = VectorParameter<float>;
using DoubleVectorParameter = VectorParameter<double>;

template <typename T> struct TypeOf;
template <> struct TypeOf<float> { static const ParameterBase::DataTypes v = ParameterBase::FLOAT; };
template <> struct TypeOf<double> { static const ParameterBase::DataTypes v = ParameterBase::DOUBLE; };
template <> struct TypeOf<int> { static const ParameterBase::DataTypes v = ParameterBase::INT32; };
template <> struct TypeOf<unsigned int> { static const ParameterBase::DataTypes v = ParameterBase::UINT32; };
template <> struct TypeOf<short> { static const ParameterBase::DataTypes v = ParameterBase::INT16; };
template <> struct TypeOf<unsigned short> { static const ParameterBase::DataTypes v = ParameterBase::UINT16; };
template <> struct TypeOf<char> { static const ParameterBase::DataTypes v = ParameterBase::INT8; };
template <> struct TypeOf<unsigned char> { static const ParameterBase::DataTypes v = ParameterBase::UINT8; };

class ParameterObject {
 public:
  virtual ~ParameterObject() {}
  virtual void initParameters() {}

  template <typename T>
  int createNumericParameter(const std::string &name, const std::string &label, T *p) {
    return add(new NumericParameter<T>(name, label, TypeOf<T>::v, p));
  }
  template <typename T>
  int createNumericParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<T> g,
                             ParameterBase::SetFunc<T> s = {}) {
    return add(new NumericParameter<T>(name, label, TypeOf<T>::v, g, s));
  }
  int createBoolParameter(const std::string &name, const std::string &label, bool *p) {
    return add(new BoolParameter(name, label, ParameterBase::BOOL, p));
  }
  int createBoolParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<bool> g,
                          ParameterBase::SetFunc<bool> s = {}) {
    return add(new BoolParameter(name, label, ParameterBase::BOOL, g, s));
  }
  int createEnumParameter(const std::string &name, const std::string &label, int *p) {
    return add(new EnumParameter(name, label, ParameterBase::ENUM, p));
  }
  int createEnumParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<int> g,
                          ParameterBase::SetFunc<int> s = {}) {
    return add(new EnumParameter(name, label, ParameterBase::ENUM, g, s));
  }
  int createStringParameter(const std::string &name, const std::string &label, std::string *p) {
    return add(new StringParameter(name, label, ParameterBase::STRING, p));
  }
  int createStringParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<std::string> g,
                            ParameterBase::SetFunc<std::string> s = {}) {
    return add(new StringParameter(name, label, ParameterBase::STRING, g, s));
  }
  template <typename T>
  int createVectorParameter(const std::string &name, const std::string &label, unsigned int dim, T *p) {
    return add(new VectorParameter<T>(name, label, sizeof(T) == 8 ? ParameterBase::VEC_DOUBLE : ParameterBase::VEC_FLOAT,
                                      dim, p));
  }
  template <typename T>
  int createVectorParameter(const std::string &name, const std::string &label, unsigned int dim,
                            ParameterBase::GetVecFunc<T> g, ParameterBase::SetVecFunc<T> s = {}) {
    return add(new VectorParameter<T>(name, label, sizeof(T) == 8 ? ParameterBase::VEC_DOUBLE : ParameterBase::VEC_FLOAT,
                                      dim, g, s));
  }

  unsigned int numParameters() const { return (unsigned int)m_params.size(); }
  void setGroup(unsigned int id, const std::string &g) { getParameter(id)->setGroup(g); }
  void setDescription(unsigned int id, const std::string &d) { getParameter(id)->setDescription(d); }
  void setReadOnly(unsigned int id, bool v) { getParameter(id)->setReadOnly(v); }
  void setVisible(unsigned int id, bool v) { getParameter(id)->setVisible(v); }
  ParameterBase *getParameter(unsigned int id) const { return m_params.at(id).get(); }
  ParameterBase *getParameter(const std::string &name) const {
    for (auto &p : m_params)
      if (p->getName() == name) return p.get();
    return nullptr;
  }
  int getParameterIndex(const std::string &name) const {
    for (size_t k = 0; k < m_params.size(); k++)
      if (m_params[k]->getName() == name) return (int)k;
    return -1;
  }

  template <typename T>
  T getValue(unsigned int id) const {
    auto *p = dynamic_cast<Parameter<T> *>(getParameter(id));
    if (!p) throw std::runtime_error("parameter type mismatch: " + getParameter(id)->getName());
    return p->getValue();
  }
  template <typename T>
  void setValue(unsigned int id, T v) {
    auto *p = dynamic_cast<Parameter<T> *>(getParameter(id));
    if (!p) throw std::runtime_error("parameter type mismatch: " + getParameter(id)->getName());
    p->setValue(v);
  }
  template <typename T>
  T *getVecValue(unsigned int id) const {
    auto *p = dynamic_cast<VectorParameter<T> *>(getParameter(id));
    if (!p) throw std::runtime_error("vector parameter type mismatch: " + getParameter(id)->getName());
    return p->getValue();
  }
  template <typename T>
  void setVecValue(unsigned int id, T *v) {
    auto *p = dynamic_cast<VectorParameter<T> *>(getParameter(id));
    if (!p) throw std::runtime_error("vector parameter type mismatch: " + getParameter(id)->getName());
    p->setValue(v);
  }

 protected:
  int add(ParameterBase *p) {
    m_params.emplace_back(p);
    return (int)m_params.size() - 1;
  }
  std::vector<std::unique_ptr<ParameterBase>> m_params;
};

}  // namespace GenParam
