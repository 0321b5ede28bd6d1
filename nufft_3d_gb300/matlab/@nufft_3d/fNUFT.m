% k = obj.fNUFT(x): forward transform, image [N1 N2 N3 nc] -> samples [M nc]
% (k = H * fft3_pad(U .* x) / sqrt(nnz), fNUFT.m:2-9 of the reference).
function k = fNUFT(obj, x)
x = single(x);
if isreal(x), x = complex(x); end
k = nufft3d_mex('forward', obj.plan, x);
