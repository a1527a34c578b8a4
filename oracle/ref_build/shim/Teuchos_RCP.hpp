/* Minimal Teuchos::RCP stand-in (shared ownership pointer) so reference
 * headers that name it compile without Trilinos. Test infrastructure only. */
#ifndef XG_SHIM_TEUCHOS_RCP
#define XG_SHIM_TEUCHOS_RCP
#include <memory>
namespace Teuchos {
template <class T> class RCP {
 public:
  RCP() {}
  RCP(T* p) : p_(p) {}
  template <class U> RCP(const RCP<U>& o) : p_(o.shared()) {}
  const std::shared_ptr<T>& shared() const { return p_; }
  T* get() const { return p_.get(); }
  T* operator->() const { return p_.get(); }
  T& operator*() const { return *p_; }
  bool is_null() const { return !p_; }
 private:
  std::shared_ptr<T> p_;
};
template <class T> RCP<T> rcp(T* p) { return RCP<T>(p); }
template <class T> using RefCountPtr = RCP<T>;
}
#endif
