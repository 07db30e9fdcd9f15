// Stand-in for core/dataTypes/SmartObject.hpp:15-88 (flags only).
#pragma once
namespace NAV24 {
class SmartObject {
public:
    virtual ~SmartObject() = default;
    [[nodiscard]] virtual bool isValid() const { return mbValid; }
    virtual void setValid(bool b) { mbValid = b; }
    [[nodiscard]] bool isOptFixed() const { return mbOptFixed; }
    void setOptFixed(bool b) { mbOptFixed = b; }
protected:
    bool mbValid = true;
    bool mbOptFixed = false;
};
}  // namespace NAV24
