set output "hist_cfg1_MOTIF00006.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-34.4237:11.3578]
set yrange [0:2025]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00006.dat" using 1:2 title 'MOTIF00006 (cfg1)' with boxes
