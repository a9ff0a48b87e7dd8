// phong.frag's composite with direct lighting (vct_shade): per pixel of a
// G-buffer, every enabled light through Cook-Torrance (GGX distribution,
// Schlick-GGX geometry, Schlick Fresnel; phong.frag:225-262, 520-545) or
// Blinn-Phong (264-273), point-light range and smoothstep attenuation
// (275-301), 5-tap PCF for shadow casters (183-207, 337-342), then the
// indirect term of a previous cone trace, occlusion and the tone map
// (main, 430-520).  Compiled with --fmad=false; pow() is CUDA's powf, so
// results match the CPU restatement to rounding, not bit for bit.
#include "vct_device.cuh"

namespace vct {

namespace {

// common.glsl:1 (sic: 3.1415982).
constexpr float kPi = 3.1415982f;

struct Lighting {
    f3 diffuse, specular;
};

__device__ __forceinline__ float pow2(float x) { return x * x; }

__device__ __forceinline__ Lighting cook_torrance(f3 dc, f3 lc, f3 N, f3 V, f3 L, f3 H, float r, float m) {
    const float n_dot_l = fmaxf(0.0f, dot(N, L));
    const float n_dot_v = fmaxf(0.0f, dot(N, V));
    const float n_dot_h = fmaxf(0.0f, dot(N, H));
    const float h_dot_v = fmaxf(0.0f, dot(H, V));
    const f3 f_lambert = mk(dc.x / kPi, dc.y / kPi, dc.z / kPi);
    // D_ggxtr
    const float alpha2 = pow2(r);
    const float D = alpha2 / (kPi * pow2(pow2(n_dot_h) * (alpha2 - 1.0f) + 1.0f));
    // G_schlickggx
    const float k = pow2(r + 1.0f) / 8.0f;
    const float g1v = n_dot_v / (n_dot_v * (1.0f - k) + k);
    const float n_dot_l2 = fmaxf(0.0f, dot(N, L));
    const float g1l = n_dot_l2 / (n_dot_l2 * (1.0f - k) + k);
    const float G = g1v * g1l;
    // F0 = mix(0.04, diffuse, metallic); schlicks
    const f3 F0 = mk(0.04f * (1.0f - m) + dc.x * m, 0.04f * (1.0f - m) + dc.y * m, 0.04f * (1.0f - m) + dc.z * m);
    const float p5 = powf(1.0f - h_dot_v, 5.0f);
    const f3 F = mk(F0.x + (1.0f - F0.x) * p5, F0.y + (1.0f - F0.y) * p5, F0.z + (1.0f - F0.z) * p5);
    const float den = fmaxf(4.0f * n_dot_l * n_dot_v, 0.001f);
    const f3 fct = mk(D * G * F.x / den, D * G * F.y / den, D * G * F.z / den);
    const f3 kd = mk((1.0f - F.x) * (1.0f - m), (1.0f - F.y) * (1.0f - m), (1.0f - F.z) * (1.0f - m));
    Lighting out;
    out.diffuse = mk(lc.x * n_dot_l * kd.x * f_lambert.x, lc.y * n_dot_l * kd.y * f_lambert.y,
                     lc.z * n_dot_l * kd.z * f_lambert.z);
    out.specular = mk(lc.x * n_dot_l * fct.x, lc.y * n_dot_l * fct.y, lc.z * n_dot_l * fct.z);
    return out;
}

__device__ __forceinline__ Lighting blinn_phong(f3 dc, const LightDev& Lt, f3 N, f3 V, f3 L, float shininess,
                                                float att) {
    const float diff = fmaxf(dot(N, L), 0.0f);
    const f3 H = normalize(add(V, L));
    const float spec = powf(fmaxf(dot(N, H), 0.0f), shininess);
    Lighting out;
    out.diffuse = mk(diff * att * Lt.color.x * Lt.intensity * dc.x, diff * att * Lt.color.y * Lt.intensity * dc.y,
                     diff * att * Lt.color.z * Lt.intensity * dc.z);
    out.specular = mk(spec * att * Lt.color.x * Lt.intensity * dc.x, spec * att * Lt.color.y * Lt.intensity * dc.y,
                      spec * att * Lt.color.z * Lt.intensity * dc.z);
    return out;
}

__global__ void __launch_bounds__(256) shade_kernel(const ShadeParams P) {
    const long long n = (long long)P.width * P.height;
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < n;
         pix += (long long)gridDim.x * blockDim.x) {
        const float4 gp = __ldg(P.gpos + pix);
        if (gp.w == 0.0f) {
            P.color[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        const float4 gn = __ldg(P.gnrm + pix);
        const float4 ga = __ldg(P.galb + pix);
        const f3 Pw = mk(gp.x, gp.y, gp.z);
        const f3 N = normalize(mk(gn.x, gn.y, gn.z));
        const f3 dc = mk(ga.x, ga.y, ga.z);
        const f3 V = normalize(sub(P.eye, Pw));
        f3 dsum = mk(0.f, 0.f, 0.f), ssum = mk(0.f, 0.f, 0.f);
        for (int i = 0; i < P.nlights; ++i) {
            const LightDev& Lt = P.lights[i];
            if (!Lt.enabled) continue;
            Lighting lg = {mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f)};
            if (Lt.type == 0u) {  // calculatePointLight
                const float dist = length(sub(Lt.position, Pw));
                if (dist > Lt.range) continue;
                const float att = 1.0f - smoothstep(0.75f * Lt.range, Lt.range, dist);
                const f3 L = normalize(sub(Lt.position, Pw));
                if (P.cooktorrance) {
                    lg = cook_torrance(dc, Lt.color, N, V, L, normalize(add(V, L)), P.roughness, P.metallic);
                    lg.diffuse = mul(lg.diffuse, att);
                    lg.specular = mul(lg.specular, att);
                } else {
                    lg = blinn_phong(dc, Lt, N, V, L, P.shininess, att);
                }
            } else if (Lt.type == 1u) {  // calculateDirectionalLight
                const f3 L = Lt.neg_dir_n;
                if (P.cooktorrance)
                    lg = cook_torrance(dc, Lt.color, N, V, L, normalize(add(V, L)), P.roughness, P.metallic);
                else
                    lg = blinn_phong(dc, Lt, N, V, L, P.shininess, 1.0f);
            }
            if (Lt.shadow_caster) {
                const float sf = 1.0f - pcf5(P.shadowmap, P.sw, P.sh, P.ls, Pw);
                lg.diffuse = mul(lg.diffuse, sf);
                lg.specular = mul(lg.specular, sf);
            }
            dsum = add(dsum, lg.diffuse);
            ssum = add(ssum, lg.specular);
        }
        const f3 dl = P.enable_diffuse ? dsum : mk(0.f, 0.f, 0.f);
        const f3 sl = P.enable_specular ? ssum : mk(0.f, 0.f, 0.f);
        f3 rgb;
        if (P.enable_indirect && P.irradiance) {
            const float4 ir = __ldg(P.irradiance + pix);
            const float occ = 1.0f - clampf(ir.w, 0.0f, 1.0f);
            f3 ind = mk(ir.x, ir.y, ir.z);
            if (P.enable_reflections && P.specular) {
                const float4 sp = __ldg(P.specular + pix);
                ind = add(ind, mul(mk(sp.x, sp.y, sp.z), P.reflect_scale));
            }
            const float as = P.ambient_scale;
            ind = mk(ind.x * (as * dc.x), ind.y * (as * dc.y), ind.z * (as * dc.z));
            rgb = add(add(ind, dl), sl);
            if (P.draw_occlusion) rgb = mul(rgb, occ);
        } else {
            rgb = add(add(mul(dc, P.ambient_scale), dl), sl);
        }
        if (P.enable_postprocess) {
            const float g = 1.0f / 2.2f;
            rgb = mk(powf(rgb.x / (rgb.x + 1.0f), g), powf(rgb.y / (rgb.y + 1.0f), g), powf(rgb.z / (rgb.z + 1.0f), g));
        }
        P.color[pix] = make_float4(rgb.x, rgb.y, rgb.z, 1.0f);
    }
}

}  // namespace

void launch_shade(const ShadeParams& P, cudaStream_t s) {
    const long long n = (long long)P.width * P.height;
    long long blocks = (n + 255) / 256;
    if (blocks > 16384) blocks = 16384;
    shade_kernel<<<(unsigned)blocks, 256, 0, s>>>(P);
    note_launches(1);
}

}  // namespace vct
