set output "hist_cfg1_MOTIF00028.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-64.2603:19.5085]
set yrange [0:158573]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00028.dat" using 1:2 title 'MOTIF00028 (cfg1)' with boxes
