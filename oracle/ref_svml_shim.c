/* Test infrastructure only. Per-lane libm stand-ins for the three Intel SVML entry points that the
 * reference declares at source/math.h:21-23 and calls at math.h:352,372,420 and
 * common_shader_core.h:232-234. SVML is closed and absent here, so colour that goes through these
 * functions is compared at +-1 LSB, not bit-exactly. */
#include <immintrin.h>
#include <math.h>

__m256 _mm256_acos_ps(__m256 x) {
    float v[8];
    _mm256_storeu_ps(v, x);
    for (int i = 0; i < 8; ++i) v[i] = acosf(v[i]);
    return _mm256_loadu_ps(v);
}

__m256 _mm256_exp_ps(__m256 x) {
    float v[8];
    _mm256_storeu_ps(v, x);
    for (int i = 0; i < 8; ++i) v[i] = expf(v[i]);
    return _mm256_loadu_ps(v);
}

__m256 _mm256_pow_ps(__m256 x, __m256 y) {
    float a[8], b[8];
    _mm256_storeu_ps(a, x);
    _mm256_storeu_ps(b, y);
    for (int i = 0; i < 8; ++i) a[i] = powf(a[i], b[i]);
    return _mm256_loadu_ps(a);
}
