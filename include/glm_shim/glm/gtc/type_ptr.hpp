// glm::value_ptr for the stand-in types of <glm/glm.hpp>: the address of the first component
// (of the first column, for a matrix), as GLM's <glm/gtc/type_ptr.hpp> gives it.
#pragma once

#include <glm/glm.hpp>

namespace glm
{

template <template <class> class V, class T>
const T* value_ptr(const V<T>& v)
{
    return &v.x;
}
template <template <class> class V, class T>
T* value_ptr(V<T>& v)
{
    return &v.x;
}
inline const float* value_ptr(const mat4& m)
{
    return &m.value[0].x;
}
inline float* value_ptr(mat4& m)
{
    return &m.value[0].x;
}

} // namespace glm
