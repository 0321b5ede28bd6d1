% x = obj.aNUFT(k): adjoint transform, samples [M nc] -> image [N1 N2 N3 nc]
% (x = U .* ifft3_crop(H' * k) / sqrt(nnz), aNUFT.m:2-9 of the reference).
function x = aNUFT(obj, k)
k = single(k);
if isreal(k), k = complex(k); end
x = nufft3d_mex('adjoint', obj.plan, k);
