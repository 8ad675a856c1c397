// splat_op.js -- the splat pipeline as a differentiable op for JavaScript callers of the N-API addon:
// forward(view) renders fp32 colour and keeps what backward needs; backward(dLdRgb) returns the
// gradients of every packed attribute (the uploadGsData layout: positions, log-scales, quaternions,
// f_dc, opacity logits, f_rest). loss() is L1 + lambda (1 - SSIM) with its gradient.
import {createRequire} from "module";

const require = createRequire(import.meta.url);
const {Native} = require("./build/Release/webgs.node");

export class SplatOp {
    #native; #count = 0; #width = 0; #height = 0;

    constructor(config = {}) {
        this.#native = new Native({...config, differentiable: true});
    }

    // data = {count, packed: Float32Array(59 * count)} as renderer.uploadGsData takes it
    setScene(data, name = "scene") {
        this.#native.uploadGsData(data, name);
        this.#native.setGs(name);
        this.#count = data.count;
    }

    // viewBlock: the 176-byte uniform block (renderer.js:773-797 layout) -> Float32Array(W*H*3)
    forward(viewBlock, width, height) {
        this.#width = width;
        this.#height = height;
        const rgb = new Float32Array(width * height * 3);
        this.#native.renderRgb(viewBlock, rgb);
        return rgb;
    }

    // dL/drgb of the last forward -> dL/d(packed attributes), Float32Array(59 * count)
    backward(dLdRgb) {
        const grad = new Float32Array(this.#count * 59);
        this.#native.backward(dLdRgb, grad);
        return grad;
    }

    // {value, grad}: L1 + lambda (1 - SSIM) of rgb against target and its gradient
    loss(rgb, target, lambda = 0.2) {
        const grad = new Float32Array(rgb.length);
        const value = this.#native.loss(rgb, target, this.#width, this.#height, lambda, grad);
        return {value, grad};
    }
}
