//! `cargo test` on a machine with a GB300 and the CUDA toolkit: the crate's calls against
//! results the test computes itself (integer masses make the eq1 gather exact in any order).
use prestige_gpu::{ffi, Config, System};

/// A jittered 12 x 12 x 12 lattice, spacing 0.01, h = 1.3 spacing (deterministic jitter).
fn lattice() -> (Config, Vec<f64>, Vec<f64>, Vec<f64>, Vec<f64>) {
    let (side, dx) = (12usize, 0.01f64);
    let n = side * side * side;
    let mut pos = Vec::with_capacity(3 * n);
    let mut vel = Vec::with_capacity(3 * n);
    let mut state: u64 = 0x9e3779b97f4a7c15;
    let mut unit = move || {
        state = state.wrapping_mul(6364136223846793005).wrapping_add(1442695040888963407);
        ((state >> 11) as f64) / ((1u64 << 53) as f64) - 0.5
    };
    for k in 0..side {
        for j in 0..side {
            for i in 0..side {
                for c in [i, j, k] {
                    pos.push((c as f64 + 0.5) * dx + 0.4 * dx * unit());
                }
                for _ in 0..3 {
                    vel.push(0.1 * unit());
                }
            }
        }
    }
    let rho: Vec<f64> = (0..n).map(|_| 1000.0 * (1.0 + 0.02 * unit())).collect();
    let mass = vec![1000.0 * dx * dx * dx; n];
    let h = 1.3 * dx;
    let extent = side as f64 * dx;
    let cfg = Config::sph(3, h, 0.25 * h / 10.0).domain([-4.0 * h; 3], [extent + 4.0 * h; 3]);
    (cfg, pos, vel, rho, mass)
}

#[test]
fn eq1_over_the_neighbour_set_is_the_brute_force_gather() {
    let (cfg, pos, _, _, _) = lattice();
    let n = pos.len() / 3;
    let mut sys = System::new(&cfg, n).unwrap();
    sys.set("pos", &pos).unwrap();
    let mass: Vec<f64> = (0..n).map(|i| (i % 7) as f64 + 1.0).collect();
    sys.set("mass", &mass).unwrap();
    sys.set("force", &vec![0.0; n]).unwrap();
    sys.run_equations(&["force [i] += mass [j] ;"]).unwrap(); // token-stream text, as fuse() stores it
    let got = sys.get("force").unwrap();
    let s2 = (2.0 * cfg.0.h) * (2.0 * cfg.0.h);
    for i in 0..n {
        let mut want = 0.0;
        for j in 0..n {
            let d: f64 = (0..3).map(|c| (pos[3 * i + c] - pos[3 * j + c]).powi(2)).sum();
            if d < s2 {
                want += mass[j];
            }
        }
        assert_eq!(got[i], want, "particle {i}");
    }
}

#[test]
fn double_word_step_follows_the_ieee_step() {
    let (cfg, pos, vel, rho, mass) = lattice();
    let n = pos.len() / 3;
    let mut a = System::new(&cfg.f64_mode(ffi::PG_F64_NATIVE), n).unwrap();
    let mut b = System::new(&cfg.f64_mode(ffi::PG_F64_FAST), n).unwrap();
    for s in [&mut a, &mut b] {
        s.set("pos", &pos).unwrap();
        s.set("vel", &vel).unwrap();
        s.set("rho", &rho).unwrap();
        s.set("mass", &mass).unwrap();
        s.step(3).unwrap();
    }
    for name in ["pos", "vel", "rho"] {
        let (x, y) = (a.get(name).unwrap(), b.get(name).unwrap());
        let scale = x.iter().fold(0.0f64, |m, v| m.max(v.abs()));
        let err = x.iter().zip(&y).fold(0.0f64, |m, (p, q)| m.max((p - q).abs()));
        assert!(err <= 1e-10 * scale, "{name}: {err} of {scale}");
    }
}

#[test]
fn adjoint_matches_central_differences_in_alpha() {
    let (cfg, pos, vel, rho, mass) = lattice();
    let n = pos.len() / 3;
    let target: Vec<f64> = pos.iter().map(|x| x + 1e-4).collect();
    let loss = |alpha: f64| -> f64 {
        let mut c = cfg;
        c.0.alpha = alpha;
        let mut s = System::new(&c, n).unwrap();
        for (k, v) in [("pos", &pos), ("vel", &vel), ("rho", &rho), ("mass", &mass)] {
            s.set(k, v).unwrap();
        }
        s.step(10).unwrap();
        let x = s.get("pos").unwrap();
        x.iter().zip(&target).map(|(a, b)| (a - b) * (a - b)).sum::<f64>() / n as f64
    };
    let mut s = System::new(&cfg, n).unwrap();
    for (k, v) in [("pos", &pos), ("vel", &vel), ("rho", &rho), ("mass", &mass)] {
        s.set(k, v).unwrap();
    }
    s.forward_checkpointed(10, 4).unwrap();
    let x = s.get("pos").unwrap();
    let dl_dx: Vec<f64> = x.iter().zip(&target).map(|(a, b)| 2.0 * (a - b) / n as f64).collect();
    let g = s.backward(&dl_dx).unwrap();
    let e = 1e-6;
    let fd = (loss(cfg.0.alpha + e) - loss(cfg.0.alpha - e)) / (2.0 * e);
    assert!((g.d_alpha - fd).abs() <= 1e-5 * fd.abs(), "{} vs {}", g.d_alpha, fd);
    assert_eq!(g.d_v0.len(), 3 * n);
}

#[test]
fn errors_carry_the_library_message() {
    let (cfg, pos, _, _, _) = lattice();
    let mut sys = System::new(&cfg, pos.len() / 3).unwrap();
    let e = sys.get("no_such_field").unwrap_err();
    assert_eq!(e.status, ffi::PG_ENOTFOUND);
    assert!(!e.message.is_empty());
    let e = sys.set("pos", &[0.0; 5]).unwrap_err();
    assert_eq!(e.status, ffi::PG_EINVAL);
}
